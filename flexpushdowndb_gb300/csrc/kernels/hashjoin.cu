// Hash join build and probe on an open-addressing table.
//
// Replaces the hash table of Arrow's hashjoin exec node that
// HashJoinArrowKernel drives (fpdb-executor/src/physical/join/hashjoin/HashJoinArrowKernel.cpp:252,334)
// and the native TupleSetIndex unordered_multimap
// (fpdb-tuple/src/TupleSetIndex.cpp:44-88,238-245).
//
// Table: a power-of-two array of 64-bit slots, each (tag << 32 | build row),
// all-ones when empty, filled with one 64-bit atomicCAS per build row and
// linear probing. For 32-bit keys the tag is the key itself, so a probe
// decides a match from the slot alone; for 64-bit keys the tag is the high
// half of the hash and a tag hit is confirmed against the build key column.
// Duplicate build keys occupy separate slots (multimap semantics). A build
// may test up to four bloom filters on its key (a bloom selection folded
// into the join) and leave out the rows that fail one. Probing:
// a lane walks one probe row's run at a time, reading per step the aligned
// four-slot group (one sector) that holds the run's next slot, and takes the
// warp's next row as soon as its run ends. Matches collect per warp in
// shared memory and leave in runs of up to kStage pairs, each run taking its
// output positions with one atomic on the shared cursor: the cursor is a
// single address whose atomics the L2 serialises, so one atomic per warp
// step held a 20M-row probe to the rate of that one address.
#include "bloom.cuh"
#include "common.cuh"
#include "launch.h"

namespace gfpdb {

namespace {

// Bloom filters the build keys must pass (a backward filter of predicate
// transfer tested in the build instead of in a selection before it); a
// filter whose size or validity lives on the device is read there.
struct BuildFilters {
  const uint32_t* blocks[kJoinBuildFiltersMax];
  const uint64_t* nblocks_dev[kJoinBuildFiltersMax];
  const int32_t* valid_dev[kJoinBuildFiltersMax];
  uint32_t num_blocks[kJoinBuildFiltersMax];
  int32_t num_hashes[kJoinBuildFiltersMax];
  int32_t valid[kJoinBuildFiltersMax];
  int32_t n;
};

__global__ void __launch_bounds__(256)
    join_build_kernel(DevCol key, int64_t cap, const int64_t* n_dev, uint64_t* __restrict__ slots, uint64_t mask,
                      int key32, DevStatus* st, BuildFilters bf) {
  const int64_t n = clamp_rows(n_dev, cap);
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  int64_t my_max = 0;
  bool dup = false;
  uint32_t nblocks[kJoinBuildFiltersMax];
  bool valid[kJoinBuildFiltersMax];
#pragma unroll
  for (int f = 0; f < kJoinBuildFiltersMax; ++f) {
    valid[f] = false;
    nblocks[f] = 0;
    if (f < bf.n) {
      nblocks[f] = bf.nblocks_dev[f] ? static_cast<uint32_t>(*bf.nblocks_dev[f]) : bf.num_blocks[f];
      valid[f] = (bf.valid_dev[f] ? (*bf.valid_dev[f] != 0) : (bf.valid[f] != 0)) && nblocks[f] > 0;
    }
  }
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
    const int64_t k = load_int(key, r);
    bool pass = true;
#pragma unroll
    for (int f = 0; f < kJoinBuildFiltersMax; ++f)
      if (valid[f] && pass) {
        const uint64_t bh = bloom_hash(k);
        pass = bloom_test(bf.blocks[f] + static_cast<uint64_t>(bloom_block_of(bh, nblocks[f])) * 8, bh,
                          bf.num_hashes[f]);
      }
    if (!pass) continue;  // cannot match a probe row that passed the filter's creator
    const uint64_t h = hash_key(k);
    const uint32_t tag = key32 ? static_cast<uint32_t>(k) : static_cast<uint32_t>(h >> 32);
    const uint64_t packed = (static_cast<uint64_t>(tag) << 32) | static_cast<uint32_t>(r);
    uint64_t slot = h & mask;
    uint64_t probe = 0;
    for (; probe <= mask; ++probe) {
      const unsigned long long old = atomicCAS(reinterpret_cast<unsigned long long*>(slots + slot),
                                               static_cast<unsigned long long>(kEmptySlot),
                                               static_cast<unsigned long long>(packed));
      if (old == kEmptySlot) break;
      // A key met again on its own run: the build side has duplicates, so a
      // probe row can match several build rows.
      if (static_cast<uint32_t>(old >> 32) == tag &&
          (key32 || load_int(key, static_cast<uint32_t>(old)) == k))
        dup = true;
      slot = (slot + 1) & mask;
    }
    if (probe > mask) raise_status(st, GFPDB_ENOMEM, 10);  // table full: cannot happen at load <= 1
    if (static_cast<int64_t>(probe) > my_max) my_max = static_cast<int64_t>(probe);
  }
  // longest probe run, for diagnostics
  for (int d = 16; d > 0; d >>= 1) {
    int64_t o = __shfl_down_sync(0xffffffffu, my_max, d);
    if (o > my_max) my_max = o;
  }
  if ((threadIdx.x & 31) == 0 && my_max > 0)
    atomicMax(reinterpret_cast<unsigned long long*>(&st->aux[0]), static_cast<unsigned long long>(my_max));
  if (dup) st->aux[1] = 1;
}

// Per-warp staging of matches: (probe row, build row) pairs in shared
// memory, flushed to the output when fewer than 32 free places remain (one
// staging round adds at most 32) and once at the end.
constexpr int kProbeWarps = 8;  // 256-thread CTAs
constexpr int kStage = 512;     // staged pairs per warp

struct PairStage {
  int32_t* p;
  int32_t* b;
  int n;  // staged pairs; the same in every lane
};

__device__ __forceinline__ void stage_pairs(PairStage& sg, bool emit, int lane, int32_t prow, int32_t brow) {
  const uint32_t em = __ballot_sync(0xffffffffu, emit);
  if (emit) {
    const int at = sg.n + __popc(em & ((1u << lane) - 1u));
    sg.p[at] = prow;
    sg.b[at] = brow;
  }
  sg.n += __popc(em);
}

// Claims sg.n output positions with one atomic and hands the stage to
// write(first position, stage, lane).
template <class Write>
__device__ __forceinline__ void flush_pairs(PairStage& sg, unsigned long long* cursor, int lane, Write& write) {
  __syncwarp();
  unsigned long long at = 0;
  if (lane == 0) at = atomicAdd(cursor, static_cast<unsigned long long>(sg.n));
  at = __shfl_sync(0xffffffffu, at, 0);
  write(static_cast<int64_t>(at), sg, lane);
  __syncwarp();
  sg.n = 0;
}

// The slot value at index q (0..3) of a four-slot group held as two 16-byte
// halves.
__device__ __forceinline__ uint64_t group_slot(const ulonglong2& lo, const ulonglong2& hi, int q) {
  const unsigned long long a = (q & 1) ? lo.y : lo.x;
  const unsigned long long b = (q & 1) ? hi.y : hi.x;
  return (q & 2) ? b : a;
}

// A probe key, streamed (evict-first): each probe row is read once, and the
// L2 is better spent on the table.
__device__ __forceinline__ int64_t load_key_stream(const DevCol& c, int64_t row) {
  if (c.type == CT_I64) return __ldcs(static_cast<const long long*>(c.data) + row);
  return __ldcs(static_cast<const int*>(c.data) + row);
}

// The probe loop shared by the pair and the materialising probe.
//
// Each warp owns a contiguous range of probe rows and each lane walks one
// row's run at a time; a lane whose run has ended takes the warp's next row
// before the next step, so lanes do not sit idle behind the longest run of
// a fixed tile. The keys of the next 128 rows of the range wait in four
// registers per lane (a ring of 32-row batches, each loaded three batches
// ahead of its use), so a new row's key comes from a shuffle rather than a
// dependent load, and a step's only wait is its table read.
//
// A step reads the aligned group of four slots (one 32-byte sector) that
// holds the run's next slot: the run is the same linear probe as the
// build's, in about a quarter of the steps. In a run's first group the
// slots before its start slot are not part of it; an empty slot at or
// after the start ends the run.
template <class Write>
__device__ __forceinline__ void probe_rows(const DevCol& pkey, int64_t n, const uint64_t* __restrict__ slots,
                                           uint64_t mask, const DevCol& bkey, int key32, unsigned long long* cursor,
                                           Write& write) {
  __shared__ int32_t s_p[kProbeWarps][kStage], s_b[kProbeWarps][kStage];
  const int lane = threadIdx.x & 31;
  const uint32_t below = (1u << lane) - 1u;
  PairStage sg{s_p[threadIdx.x >> 5], s_b[threadIdx.x >> 5], 0};
  const int64_t warp_global = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  const int64_t per = ((n + n_warps - 1) / n_warps + 31) & ~static_cast<int64_t>(31);
  const int64_t begin = warp_global * per < n ? warp_global * per : n;
  const int64_t end = begin + per < n ? begin + per : n;
  // A table always keeps empty slots (load factor <= 0.9), so every run
  // ends within one pass over the groups; the bound only guards the loop.
  const uint64_t n_groups = (mask + 1) >> 2;

  int64_t ring[4];  // keys of rows ring_base + 32 * b + lane
  int64_t ring_base = begin;
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const int64_t r = begin + 32 * b + lane;
    ring[b] = r < end ? load_key_stream(pkey, r) : 0;
  }
  int taken = 0;  // rows of the ring's first batch already handed out (< 32 between steps)

  bool active = false;
  int32_t row = 0;
  int64_t k = 0;
  uint32_t tag = 0, valid = 0;
  uint64_t grp = 0, steps = 0;
  while (true) {
    // Hand the next rows of the range to the lanes without one, in lane
    // order: the lane of rank i among them takes row ring_base + taken + i.
    const uint32_t idle = __ballot_sync(0xffffffffu, !active);
    const int64_t left = end - (ring_base + taken);
    if (idle == 0xffffffffu && left <= 0) break;
    if (idle != 0 && left > 0) {
      const int idx = taken + __popc(idle & below);  // < 64: in the ring's first two batches
      const int64_t v0 = __shfl_sync(0xffffffffu, ring[0], idx & 31);
      const int64_t v1 = __shfl_sync(0xffffffffu, ring[1], idx & 31);
      if (!active && idx - taken < left) {
        active = true;
        row = static_cast<int32_t>(ring_base + idx);
        k = idx < 32 ? v0 : v1;
        const uint64_t h = hash_key(k);
        tag = key32 ? static_cast<uint32_t>(k) : static_cast<uint32_t>(h >> 32);
        const uint64_t slot = h & mask;
        grp = slot & ~3ull;
        valid = (0xFu << (slot & 3)) & 0xFu;
        steps = 0;
      }
      const int handed = static_cast<int64_t>(__popc(idle)) < left ? __popc(idle) : static_cast<int>(left);
      taken += handed;
      if (taken >= 32) {  // the first batch is used up: shift, fetch the batch after the last
        ring[0] = ring[1];
        ring[1] = ring[2];
        ring[2] = ring[3];
        const int64_t r = ring_base + 128 + lane;
        ring[3] = r < end ? load_key_stream(pkey, r) : 0;
        ring_base += 32;
        taken -= 32;
      }
    }

    uint32_t mm = 0;  // matching slots of this step's group that lie on the run
    ulonglong2 lo{0, 0}, hi{0, 0};
    if (active) {
      const ulonglong2* g = reinterpret_cast<const ulonglong2*>(slots + grp);
      lo = __ldg(g);
      hi = __ldg(g + 1);
      uint32_t eb = 0, tb = 0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint64_t v = group_slot(lo, hi, q);
        if (v == kEmptySlot)
          eb |= 1u << q;
        else if (static_cast<uint32_t>(v >> 32) == tag)
          tb |= 1u << q;
      }
      eb &= valid;
      const int stop = eb ? __ffs(eb) - 1 : 4;
      mm = tb & valid & ((1u << stop) - 1u);
      if (!key32) {
        for (uint32_t t = mm; t != 0; t &= t - 1) {
          const int q = __ffs(t) - 1;
          if (load_int(bkey, static_cast<int32_t>(static_cast<uint32_t>(group_slot(lo, hi, q)))) != k)
            mm &= ~(1u << q);
        }
      }
      if (eb != 0 || ++steps > n_groups) {
        active = false;
      } else {
        grp = (grp + 4) & mask;
        valid = 0xFu;
      }
    }
    // One staged match per lane per round; a group can hold several copies
    // of a repeated build key.
    while (__any_sync(0xffffffffu, mm != 0)) {
      int32_t brow = 0;
      const bool emit = mm != 0;
      if (emit) {
        brow = static_cast<int32_t>(static_cast<uint32_t>(group_slot(lo, hi, __ffs(mm) - 1)));
        mm &= mm - 1;
      }
      stage_pairs(sg, emit, lane, row, brow);
      if (sg.n > kStage - 32) flush_pairs(sg, cursor, lane, write);
    }
  }
  if (sg.n > 0) flush_pairs(sg, cursor, lane, write);
}

__global__ void __launch_bounds__(256)
    join_probe_kernel(DevCol pkey, int64_t n_cap, const int64_t* n_dev, const uint64_t* __restrict__ slots,
                      uint64_t mask, DevCol bkey, int key32, int32_t* __restrict__ out_p,
                      int32_t* __restrict__ out_b, int64_t cap, DevStatus* st) {
  const int64_t n = clamp_rows(n_dev, n_cap);
  auto write = [&](int64_t at, const PairStage& sg, int lane) {
    for (int i = lane; i < sg.n; i += 32)
      if (at + i < cap) {
        __stcs(out_p + at + i, sg.p[i]);
        __stcs(out_b + at + i, sg.b[i]);
      }
  };
  probe_rows(pkey, n, slots, mask, bkey, key32, reinterpret_cast<unsigned long long*>(&st->value), write);
}

// Probe and materialise in one pass: every staged match becomes an output
// row (probe columns from the probe row, build columns from the build row)
// at the positions its flush claimed, so no pair buffer and no separate
// gather launch are needed. Fixed-width columns only.
constexpr int kJoinOutMax = 24;

struct JoinEmitParams {
  DevCol pkey;
  DevCol bkey;
  int64_t n_cap;
  const int64_t* n_dev;
  const uint64_t* slots;
  uint64_t mask;
  int64_t cap;
  DevStatus* st;
  int32_t key32;
  int32_t n_out;
  const void* src[kJoinOutMax];
  void* dst[kJoinOutMax];
  int32_t width[kJoinOutMax];
  int32_t from_build[kJoinOutMax];
};

// One column of a flush: four gathers in flight per lane, then the stores,
// which stream (evict-first): the output is written once and read by later
// kernels, while the L2 should keep the hash table and the build columns
// that the probes and gathers revisit.
template <class T>
__device__ __forceinline__ void copy_staged(const T* __restrict__ src, T* __restrict__ dst, const int32_t* idx,
                                            int n, int64_t at, int64_t cap, int lane, bool stream_src) {
  constexpr int kU = 4;
  for (int i0 = 0; i0 < n; i0 += 32 * kU) {
    T v[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int i = i0 + u * 32 + lane;
      if (i < n) v[u] = stream_src ? __ldcs(src + idx[i]) : __ldg(src + idx[i]);
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int i = i0 + u * 32 + lane;
      if (i < n && at + i < cap) __stcs(dst + at + i, v[u]);
    }
  }
}

__global__ void __launch_bounds__(256) join_probe_emit_kernel(const __grid_constant__ JoinEmitParams p) {
  const int64_t n = clamp_rows(p.n_dev, p.n_cap);
  auto write = [&](int64_t at, const PairStage& sg, int lane) {
    for (int c = 0; c < p.n_out; ++c) {
      const int32_t* idx = p.from_build[c] ? sg.b : sg.p;
      // probe rows are read once (streamed); build rows are revisited
      const bool stream_src = !p.from_build[c];
      if (p.width[c] == 8)
        copy_staged(static_cast<const long long*>(p.src[c]), static_cast<long long*>(p.dst[c]), idx, sg.n, at, p.cap,
                    lane, stream_src);
      else
        copy_staged(static_cast<const int*>(p.src[c]), static_cast<int*>(p.dst[c]), idx, sg.n, at, p.cap, lane,
                    stream_src);
    }
  };
  probe_rows(p.pkey, n, p.slots, p.mask, p.bkey, p.key32, reinterpret_cast<unsigned long long*>(&p.st->value), write);
}

// A chain of joins in one pass. Each lane walks its input row through the
// levels like a depth-first search: at its current level it reads, per
// step, the aligned four-slot group holding its run's next slot (and knows
// the run is over, without another read, when an empty slot follows the
// match in that group); a match at an inner level moves it to the next level (whose key
// comes from the input row or an earlier match), a match at the last level
// emits an output row, and the end of a run returns it to the level before,
// whose run it continues. The warp steps together so that emitted rows can
// be staged with one ballot per step.
struct ChainLevel {
  const uint64_t* slots;
  uint64_t mask;
  DevCol bkey;         // the level's build key column (confirms 64-bit keys)
  const void* key;     // the level's probe key column
  int32_t key_src;     // 0: the input row; l + 1: the build row matched at level l
  int32_t key_wide;    // 1: int64 probe key column
  int32_t key32;       // 1: the slot tag is the key itself
  int32_t pad;
};

struct ChainParams {
  int64_t n_cap;
  const int64_t* n_dev;
  int32_t n_levels;
  int32_t n_out;
  int64_t cap;
  DevStatus* st;
  ChainLevel lv[kJoinChainMax];
  const void* src[kJoinOutMax];
  void* dst[kJoinOutMax];
  int32_t width[kJoinOutMax];
  int32_t from[kJoinOutMax];  // 0: the input row; l + 1: the build row of level l
};

// kStaged: output rows collect per warp in shared memory as the row index of
// every level (input row, then each join's build row) and leave in runs,
// each run taking its positions with one atomic on the shared cursor (for
// large inputs, whose per-step atomics would queue on that one address).
// Otherwise a warp step's rows are written at once with one atomic per step
// (small inputs, where the final flush would only add a round trip).
constexpr int kChainStage = 128;
constexpr int64_t kChainStagedRows = 1 << 20;

template <bool kStaged>
__global__ void __launch_bounds__(256) join_chain_kernel(const __grid_constant__ ChainParams p) {
  const int64_t n = clamp_rows(p.n_dev, p.n_cap);
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int64_t warp_global = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  unsigned long long* cursor = reinterpret_cast<unsigned long long*>(&p.st->value);
  __shared__ int32_t s_rows[kStaged ? kProbeWarps : 1][kJoinChainMax + 1][kStaged ? kChainStage : 1];
  int staged = 0;  // the same in every lane
  auto flush = [&]() {
    __syncwarp();
    unsigned long long at = 0;
    if (lane == 0) at = atomicAdd(cursor, static_cast<unsigned long long>(staged));
    at = __shfl_sync(0xffffffffu, at, 0);
    for (int c = 0; c < p.n_out; ++c) {
      const int32_t* idx = s_rows[warp][p.from[c]];
      const bool stream_src = p.from[c] == 0;  // the input row: read once
      if (p.width[c] == 8)
        copy_staged(static_cast<const long long*>(p.src[c]), static_cast<long long*>(p.dst[c]), idx, staged,
                    static_cast<int64_t>(at), p.cap, lane, stream_src);
      else
        copy_staged(static_cast<const int*>(p.src[c]), static_cast<int*>(p.dst[c]), idx, staged,
                    static_cast<int64_t>(at), p.cap, lane, stream_src);
    }
    __syncwarp();
    staged = 0;
  };
  for (int64_t base = warp_global * 32; base < n; base += n_warps * 32) {
    const int64_t r = base + lane;
    bool active = r < n;
    int64_t rows[kJoinChainMax + 1];
    uint64_t slot[kJoinChainMax], steps[kJoinChainMax];
    int64_t key[kJoinChainMax];
    uint32_t tag[kJoinChainMax];
    int lvl = 0;
    uint32_t ended = 0;  // levels whose run is known to have ended
    rows[0] = r;
    auto start_level = [&](int l) {
      const ChainLevel& L = p.lv[l];
      const int64_t kr = rows[L.key_src];
      const int64_t k = L.key_wide ? static_cast<int64_t>(__ldg(static_cast<const long long*>(L.key) + kr))
                                   : static_cast<int64_t>(__ldg(static_cast<const int*>(L.key) + kr));
      const uint64_t h = hash_key(k);
      key[l] = k;
      tag[l] = L.key32 ? static_cast<uint32_t>(k) : static_cast<uint32_t>(h >> 32);
      slot[l] = h & L.mask;
      steps[l] = 0;
      ended &= ~(1u << l);
    };
    if (active) start_level(0);
    while (__any_sync(0xffffffffu, active)) {
      bool emit = false;
      if (active) {
        const ChainLevel& L = p.lv[lvl];
        bool run_over = (ended >> lvl & 1u) != 0;
        if (!run_over) {
          // the aligned four-slot group (one sector) holding the run's next
          // slot: the first match at or after it that precedes an empty slot
          const uint64_t s0 = slot[lvl];
          const int q0 = static_cast<int>(s0 & 3);
          const uint64_t g = s0 & ~3ull;
          const ulonglong2* gp = reinterpret_cast<const ulonglong2*>(L.slots + g);
          const ulonglong2 lo = __ldg(gp), hi = __ldg(gp + 1);
          uint32_t eb = 0, tb = 0;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const uint64_t v = group_slot(lo, hi, q);
            if (v == kEmptySlot)
              eb |= 1u << q;
            else if (static_cast<uint32_t>(v >> 32) == tag[lvl])
              tb |= 1u << q;
          }
          const uint32_t from = (0xFu << q0) & 0xFu;
          eb &= from;
          const int stop = eb ? __ffs(eb) - 1 : 4;
          tb &= from & ((1u << stop) - 1u);
          int m = -1;
          int32_t brow = 0;
          for (; tb != 0; tb &= tb - 1) {
            const int q = __ffs(tb) - 1;
            const int32_t b = static_cast<int32_t>(static_cast<uint32_t>(group_slot(lo, hi, q)));
            if (L.key32 || load_int(L.bkey, b) == key[lvl]) {
              m = q;
              brow = b;
              break;
            }
          }
          steps[lvl] += static_cast<uint64_t>(4 - q0);
          if (m >= 0) {
            slot[lvl] = (g + m + 1) & L.mask;
            // the run ends in this group when an empty slot follows the
            // match with no other candidate (a repeated key) before it; tb
            // still holds the match and the candidates after it
            if (eb != 0 && (tb >> (m + 1)) == 0) ended |= 1u << lvl;
            rows[lvl + 1] = brow;
            if (lvl == p.n_levels - 1) {
              emit = true;  // and the last level's run continues next step
            } else {
              ++lvl;
              start_level(lvl);
            }
          } else if (eb != 0 || steps[lvl] > L.mask + 1) {
            run_over = true;
          } else {
            slot[lvl] = (g + 4) & L.mask;
          }
        }
        if (run_over) {
          if (lvl == 0) active = false;  // the input row is done
          else --lvl;                    // back to the previous level's run
        }
      }
      const uint32_t em = __ballot_sync(0xffffffffu, emit);
      if constexpr (kStaged) {
        if (emit) {
          const int at = staged + __popc(em & ((1u << lane) - 1u));
          for (int l = 0; l <= p.n_levels; ++l) s_rows[warp][l][at] = static_cast<int32_t>(rows[l]);
        }
        staged += __popc(em);
        if (staged > kChainStage - 32) flush();
      } else if (em != 0) {
        unsigned long long at = 0;
        const int leader = __ffs(em) - 1;
        if (lane == leader) at = atomicAdd(cursor, static_cast<unsigned long long>(__popc(em)));
        at = __shfl_sync(0xffffffffu, at, leader);
        if (emit) {
          const int64_t pos = static_cast<int64_t>(at) + __popc(em & ((1u << lane) - 1u));
          if (pos < p.cap) {
            // four output columns per round: their gathers in flight
            // together, then the stores
            for (int c0 = 0; c0 < p.n_out; c0 += 4) {
              long long v[4];
#pragma unroll
              for (int j = 0; j < 4; ++j) {
                const int c = c0 + j;
                if (c < p.n_out) {
                  const int64_t from = rows[p.from[c]];
                  v[j] = p.width[c] == 8 ? __ldg(static_cast<const long long*>(p.src[c]) + from)
                                         : static_cast<long long>(__ldg(static_cast<const int*>(p.src[c]) + from));
                }
              }
#pragma unroll
              for (int j = 0; j < 4; ++j) {
                const int c = c0 + j;
                if (c >= p.n_out) break;
                if (p.width[c] == 8)
                  static_cast<long long*>(p.dst[c])[pos] = v[j];
                else
                  static_cast<int*>(p.dst[c])[pos] = static_cast<int>(v[j]);
              }
            }
          }
        }
      }
    }
  }
  if (kStaged && staged > 0) flush();
}

// Grid-stride launches: four CTAs per SM keep the build's atomics busy, and
// a launch sized for a large row capacity of which few rows arrive
// (deferred inputs) dispatches fewer empty CTAs.
int grid_for(int64_t n, int per_sm = 4, int64_t rows_per_block = 256) {
  int64_t blocks = (n + rows_per_block - 1) / rows_per_block;
  int64_t cap = static_cast<int64_t>(num_sms()) * per_sm;
  if (blocks > cap) blocks = cap;
  return static_cast<int>(blocks < 1 ? 1 : blocks);
}

// The probes' warps wait on table loads, so their grids fill every SM with
// as many CTAs as fit at once (one wave, no tail).
template <class Kernel>
int probe_grid(Kernel kernel, int64_t n) {
  static const int per_sm = [kernel] {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, 256, 0) != cudaSuccess || b < 1) b = 4;
    return b;
  }();
  return grid_for(n, per_sm, kProbeWarps * 256);  // at least 256 rows per warp
}

}  // namespace

void join_build_table(JoinTable& t, double load_factor, cudaStream_t s, const std::vector<BloomPtr>& filters) {
  if (filters.size() > static_cast<size_t>(kJoinBuildFiltersMax))
    fail(GFPDB_EUNSUPPORTED, "a hash join build tests at most 4 bloom filters");
  if (!(load_factor > 0.0 && load_factor <= 0.9)) fail(GFPDB_EINVAL, "hash join load factor must be in (0, 0.9]");
  const int64_t n = t.build->num_rows();
  if (n >= INT32_MAX) fail(GFPDB_EUNSUPPORTED, "hash join build side must have fewer than 2^31 rows");
  uint64_t cap = 64;
  while (static_cast<double>(cap) * load_factor < static_cast<double>(n)) cap <<= 1;
  t.capacity = cap;
  t.slots = make_filled(static_cast<int64_t>(cap) * 8, 0xFF, s);
  t.status = make_filled(sizeof(DevStatus), 0, s);
  DevStatus* st = t.status->as<DevStatus>();
  const auto& kc = t.build->column(t.key_col);
  t.key_type = kc->type;
  if (n > 0) {
    DevCol k{kc->data, nullptr, static_cast<int32_t>(kc->type), 0};
    const int key32 = kc->type != DType::Int64;
    if (!filters.empty() && (kc->type == DType::Utf8 || kc->type == DType::Float64))
      fail(GFPDB_EUNSUPPORTED, "bloom filters tested in a hash join build need an integer key");
    BuildFilters bf{};
    bf.n = static_cast<int32_t>(filters.size());
    for (size_t f = 0; f < filters.size(); ++f) {
      const BloomFilterDev& b = *filters[f];
      if (b.num_blocks >= (int64_t{1} << 32)) fail(GFPDB_EUNSUPPORTED, "bloom filter too large");
      bf.blocks[f] = b.blocks ? b.blocks->as<uint32_t>() : nullptr;
      bf.nblocks_dev[f] = b.nblocks_dev;
      bf.valid_dev[f] = b.valid_dev;
      bf.num_blocks[f] = static_cast<uint32_t>(b.num_blocks);
      bf.num_hashes[f] = b.num_hashes;
      bf.valid[f] = (b.valid && bf.blocks[f] != nullptr) ? 1 : 0;
      if (bf.blocks[f] == nullptr) bf.valid_dev[f] = nullptr;
    }
    ProfScope prof("join_build_kernel", s);
    join_build_kernel<<<grid_for(n), 256, 0, s>>>(k, n, t.build->rows_dev(), t.slots->as<uint64_t>(), cap - 1,
                                                 key32, st, bf);
    after_launch("join_build_kernel");
    prof.stop(static_cast<double>(n) * dtype_width(kc->type));
  }
}

std::vector<ColumnPtr> join_probe_materialize(const JoinTable& t, const TupleSet& probe, int probe_key,
                                              const std::vector<int>& probe_cols, const std::vector<int>& build_cols,
                                              int64_t* n_out, cudaStream_t s, BufferPtr* count_owner,
                                              const int64_t** count_dev) {
  const int64_t n = probe.num_rows();
  if (n >= INT32_MAX) fail(GFPDB_EUNSUPPORTED, "hash join probe batch must have fewer than 2^31 rows");
  const auto& pc = probe.column(probe_key);
  if (pc->type == DType::Utf8 || pc->type == DType::Float64)
    fail(GFPDB_EUNSUPPORTED, "hash join keys must be integer columns");
  const bool key32 = t.key_type != DType::Int64 && pc->type != DType::Int64;
  if (!key32 && t.key_type != DType::Int64)
    fail(GFPDB_EUNSUPPORTED, "int64 probe key against an int32 build key");
  if (probe_cols.size() + build_cols.size() > static_cast<size_t>(kJoinOutMax))
    fail(GFPDB_EUNSUPPORTED, "too many hash join output columns");
  const auto& bk = t.build->column(t.key_col);
  JoinEmitParams p{};
  p.pkey = DevCol{pc->data, nullptr, static_cast<int32_t>(pc->type), 0};
  p.bkey = DevCol{bk->data, nullptr, static_cast<int32_t>(bk->type), 0};
  p.n_cap = n;
  p.n_dev = probe.rows_dev();
  p.slots = t.slots->as<uint64_t>();
  p.mask = t.capacity - 1;
  p.key32 = key32 ? 1 : 0;
  std::vector<const Column*> srcs;
  std::vector<int> from_build;
  for (int c : probe_cols) {
    srcs.push_back(probe.column(c).get());
    from_build.push_back(0);
  }
  for (int c : build_cols) {
    srcs.push_back(t.build->column(c).get());
    from_build.push_back(1);
  }
  p.n_out = static_cast<int32_t>(srcs.size());
  auto status = make_filled(sizeof(DevStatus), 0, s);
  const bool defer = deferred_mode() && count_dev != nullptr;
  int64_t cap = n > 0 ? n : 1;
  std::vector<BufferPtr> bufs(srcs.size());
  for (int attempt = 0; attempt < 2; ++attempt) {
    for (size_t c = 0; c < srcs.size(); ++c) {
      if (srcs[c]->type == DType::Utf8) fail(GFPDB_EUNSUPPORTED, "utf8 output in the fused join");
      const int w = dtype_width(srcs[c]->type);
      bufs[c] = make_buffer(cap * w, s);
      p.src[c] = srcs[c]->data;
      p.dst[c] = bufs[c]->data();
      p.width[c] = w;
      p.from_build[c] = from_build[c];
    }
    p.cap = cap;
    p.st = status->as<DevStatus>();
    if (attempt > 0) GF_CUDA(cudaMemsetAsync(status->data(), 0, sizeof(DevStatus), s));
    if (n > 0 && t.build->num_rows() > 0) {
      ProfScope prof("join_probe_emit_kernel", s);
      join_probe_emit_kernel<<<probe_grid(join_probe_emit_kernel, n), 256, 0, s>>>(p);
      after_launch("join_probe_emit_kernel");
      prof.stop(0);
      double w_out = 0;
      for (size_t c = 0; c < srcs.size(); ++c) w_out += 2.0 * p.width[c];
      prof.set_bytes_model(probe.rows_dev(), n, dtype_width(pc->type), &status->as<DevStatus>()->value, w_out, status,
                           probe.rows_owner());
    }
    if (defer) {
      defer_check(status, status->as<DevStatus>(), "hash join probe", cap);
      *n_out = cap;
      *count_dev = &status->as<DevStatus>()->value;
      if (count_owner) *count_owner = status;
      break;
    }
    DevStatus hs;
    GF_CUDA(cudaMemcpyAsync(&hs, status->data(), sizeof(hs), cudaMemcpyDeviceToHost, s));
    sync(s);
    raise_device_status(hs, "hash join probe");
    if (hs.value <= cap) {
      *n_out = hs.value;
      break;
    }
    cap = hs.value;  // more matches than probe rows (repeated build keys): once more, exactly sized
  }
  std::vector<ColumnPtr> cols;
  for (size_t c = 0; c < srcs.size(); ++c) cols.push_back(make_fixed_column(srcs[c]->type, *n_out, bufs[c]));
  return cols;
}

std::vector<ColumnPtr> join_chain_materialize(const std::vector<const JoinTable*>& tables, const TupleSet& probe,
                                              const std::vector<ChainRef>& keys, const std::vector<ChainRef>& outs,
                                              int64_t* n_out, cudaStream_t s, BufferPtr* count_owner,
                                              const int64_t** count_dev) {
  const int L = static_cast<int>(tables.size());
  if (L < 1 || L > kJoinChainMax) fail(GFPDB_EUNSUPPORTED, "a join chain has 1 to 6 joins");
  if (static_cast<int>(keys.size()) != L) fail(GFPDB_EINVAL, "a join chain needs one probe key per join");
  if (outs.size() > static_cast<size_t>(kJoinOutMax)) fail(GFPDB_EUNSUPPORTED, "too many hash join output columns");
  const int64_t n = probe.num_rows();
  if (n >= INT32_MAX) fail(GFPDB_EUNSUPPORTED, "hash join probe batch must have fewer than 2^31 rows");
  auto source = [&](int src) -> const TupleSet& { return src == 0 ? probe : *tables[src - 1]->build; };
  ChainParams p{};
  p.n_cap = n;
  p.n_dev = probe.rows_dev();
  p.n_levels = L;
  bool empty_build = false;
  for (int l = 0; l < L; ++l) {
    const JoinTable& t = *tables[l];
    if (keys[l].src < 0 || keys[l].src > l) fail(GFPDB_EINVAL, "a join chain key comes from the input or an earlier join");
    const auto& kc = source(keys[l].src).column(keys[l].col);
    if (kc->type == DType::Utf8 || kc->type == DType::Float64)
      fail(GFPDB_EUNSUPPORTED, "hash join keys must be integer columns");
    const bool key32 = t.key_type != DType::Int64 && kc->type != DType::Int64;
    if (!key32 && t.key_type != DType::Int64)
      fail(GFPDB_EUNSUPPORTED, "int64 probe key against an int32 build key");
    const auto& bk = t.build->column(t.key_col);
    ChainLevel& lv = p.lv[l];
    lv.slots = t.slots->as<uint64_t>();
    lv.mask = t.capacity - 1;
    lv.bkey = DevCol{bk->data, nullptr, static_cast<int32_t>(bk->type), 0};
    lv.key = kc->data;
    lv.key_src = keys[l].src;
    lv.key_wide = kc->type == DType::Int64 ? 1 : 0;
    lv.key32 = key32 ? 1 : 0;
    empty_build |= t.build->num_rows() == 0;
  }
  std::vector<const Column*> srcs;
  for (auto& o : outs) {
    if (o.src < 0 || o.src > L) fail(GFPDB_EINVAL, "a join chain output comes from the input or one of its joins");
    const Column* c = source(o.src).column(o.col).get();
    if (c->type == DType::Utf8) fail(GFPDB_EUNSUPPORTED, "utf8 output in the fused join");
    srcs.push_back(c);
  }
  p.n_out = static_cast<int32_t>(srcs.size());
  auto status = make_filled(sizeof(DevStatus), 0, s);
  const bool defer = deferred_mode() && count_dev != nullptr;
  int64_t cap = n > 0 ? n : 1;
  std::vector<BufferPtr> bufs(srcs.size());
  for (int attempt = 0; attempt < 2; ++attempt) {
    for (size_t c = 0; c < srcs.size(); ++c) {
      const int w = dtype_width(srcs[c]->type);
      bufs[c] = make_buffer(cap * w, s);
      p.src[c] = srcs[c]->data;
      p.dst[c] = bufs[c]->data();
      p.width[c] = w;
      p.from[c] = outs[c].src;
    }
    p.cap = cap;
    p.st = status->as<DevStatus>();
    if (attempt > 0) GF_CUDA(cudaMemsetAsync(status->data(), 0, sizeof(DevStatus), s));
    if (n > 0 && !empty_build) {
      ProfScope prof("join_chain_kernel", s);
      if (n >= kChainStagedRows)
        join_chain_kernel<true><<<grid_for(n), 256, 0, s>>>(p);
      else
        join_chain_kernel<false><<<grid_for(n), 256, 0, s>>>(p);
      after_launch("join_chain_kernel");
      prof.stop(0);
      double w_out = 0;
      for (size_t c = 0; c < srcs.size(); ++c) w_out += 2.0 * p.width[c];
      prof.set_bytes_model(probe.rows_dev(), n, dtype_width(source(keys[0].src).column(keys[0].col)->type),
                           &status->as<DevStatus>()->value, w_out, status, probe.rows_owner());
    }
    if (defer) {
      defer_check(status, status->as<DevStatus>(), "hash join chain probe", cap);
      *n_out = cap;
      *count_dev = &status->as<DevStatus>()->value;
      if (count_owner) *count_owner = status;
      break;
    }
    DevStatus hs;
    GF_CUDA(cudaMemcpyAsync(&hs, status->data(), sizeof(hs), cudaMemcpyDeviceToHost, s));
    sync(s);
    raise_device_status(hs, "hash join chain probe");
    if (hs.value <= cap) {
      *n_out = hs.value;
      break;
    }
    cap = hs.value;  // more combinations than input rows (repeated build keys): once more, exactly sized
  }
  std::vector<ColumnPtr> cols;
  for (size_t c = 0; c < srcs.size(); ++c) cols.push_back(make_fixed_column(srcs[c]->type, *n_out, bufs[c]));
  return cols;
}

void join_probe_pairs(const JoinTable& t, const TupleSet& probe, int probe_key, BufferPtr* probe_idx,
                      BufferPtr* build_idx, int64_t* n_out, cudaStream_t s, BufferPtr* count_owner,
                      const int64_t** count_dev) {
  const int64_t n = probe.num_rows();
  if (n >= INT32_MAX) fail(GFPDB_EUNSUPPORTED, "hash join probe batch must have fewer than 2^31 rows");
  const auto& pc = probe.column(probe_key);
  if (pc->type == DType::Utf8 || pc->type == DType::Float64)
    fail(GFPDB_EUNSUPPORTED, "hash join keys must be integer columns");
  // A 32-bit build key stores the key as the tag; a 64-bit probe key must
  // then also fit 32 bits to match, which the tag comparison handles because
  // the tag is the low 32 bits of the sign-extended value and the full value
  // is compared below when either side is 64-bit.
  const bool key32 = t.key_type != DType::Int64 && pc->type != DType::Int64;
  if (!key32 && t.key_type != DType::Int64)
    fail(GFPDB_EUNSUPPORTED, "int64 probe key against an int32 build key");
  const auto& bk = t.build->column(t.key_col);
  DevCol pk{pc->data, nullptr, static_cast<int32_t>(pc->type), 0};
  DevCol bkc{bk->data, nullptr, static_cast<int32_t>(bk->type), 0};
  int64_t cap = n > 0 ? n : 1;
  auto status = make_filled(sizeof(DevStatus), 0, s);
  const bool defer = deferred_mode() && count_dev != nullptr;
  for (int attempt = 0; attempt < 2; ++attempt) {
    *probe_idx = make_buffer(cap * 4, s);
    *build_idx = make_buffer(cap * 4, s);
    if (attempt > 0) GF_CUDA(cudaMemsetAsync(status->data(), 0, sizeof(DevStatus), s));
    if (n > 0 && t.build->num_rows() > 0) {
      ProfScope prof("join_probe_kernel", s);
      join_probe_kernel<<<probe_grid(join_probe_kernel, n), 256, 0, s>>>(pk, n, probe.rows_dev(), t.slots->as<uint64_t>(),
                                                   t.capacity - 1, bkc, key32 ? 1 : 0, (*probe_idx)->as<int32_t>(),
                                                   (*build_idx)->as<int32_t>(), cap, status->as<DevStatus>());
      after_launch("join_probe_kernel");
      prof.stop(static_cast<double>(n) * dtype_width(pc->type));
      prof.set_bytes_model(probe.rows_dev(), n, dtype_width(pc->type), &status->as<DevStatus>()->value, 8.0, status,
                           probe.rows_owner());
    }
    if (defer) {
      // The pairs fit whenever the build keys are unique; the plan's final
      // checks re-run it with exact sizes if they did not.
      defer_check(status, status->as<DevStatus>(), "hash join probe", cap);
      *n_out = cap;
      *count_dev = &status->as<DevStatus>()->value;
      if (count_owner) *count_owner = status;
      return;
    }
    DevStatus hs;
    GF_CUDA(cudaMemcpyAsync(&hs, status->data(), sizeof(hs), cudaMemcpyDeviceToHost, s));
    sync(s);
    raise_device_status(hs, "hash join probe");
    if (hs.value <= cap) {
      *n_out = hs.value;
      return;
    }
    if (hs.value >= INT32_MAX) fail(GFPDB_EUNSUPPORTED, "hash join output exceeds 2^31 rows");
    cap = hs.value;  // many-to-many: rerun with the exact output size
  }
  fail(GFPDB_EDEVICE, "hash join output size changed between passes");
}

// ------------------------------------------------------ outer and semi joins
//
// The non-inner join types of HashJoinArrowKernel
// (fpdb-executor/src/physical/join/hashjoin/HashJoinArrowKernel.cpp:164-195)
// on the same table: one pass counts each probe row's matches (and can mark
// the build rows it matched), a prefix sum places every probe row's output,
// and a second pass writes the (probe row, build row) pairs in probe-row
// order, a probe row without a match as (row, -1) when it is kept (a null
// build side). Marked or unmarked build rows are then listed by rows_where.

namespace {

struct MatchParams {
  DevCol pkey, bkey;
  const uint64_t* slots;
  uint64_t mask;
  int32_t key32;
  int32_t keep_unmatched;  // a probe row without a match still takes one output pair
  int64_t n;
  int32_t* counts;         // output pairs of each probe row, or null
  int32_t* matched;        // 1 at each build row some probe row matched, or null
  const int32_t* offs;     // emit: first output pair of each probe row
  int32_t* out_p;
  int32_t* out_b;
};

// Calls f(build row, j) for the j-th match of probe row r; returns the matches.
template <class F>
__device__ __forceinline__ int walk_matches(const MatchParams& p, int64_t r, F&& f) {
  const int64_t k = load_int(p.pkey, r);
  const uint64_t h = hash_key(k);
  const uint32_t tag = p.key32 ? static_cast<uint32_t>(k) : static_cast<uint32_t>(h >> 32);
  uint64_t slot = h & p.mask;
  int m = 0;
  for (uint64_t i = 0; i <= p.mask; ++i, slot = (slot + 1) & p.mask) {
    const uint64_t s = __ldg(p.slots + slot);
    if (s == kEmptySlot) break;
    if (static_cast<uint32_t>(s >> 32) != tag) continue;
    const uint32_t b = static_cast<uint32_t>(s);
    if (!p.key32 && load_int(p.bkey, b) != k) continue;
    f(b, m);
    ++m;
  }
  return m;
}

__global__ void __launch_bounds__(256) join_match_kernel(const __grid_constant__ MatchParams p) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < p.n; r += stride) {
    const int m = walk_matches(p, r, [&](uint32_t b, int) {
      if (p.matched != nullptr) p.matched[b] = 1;
    });
    if (p.counts != nullptr) p.counts[r] = (p.keep_unmatched && m == 0) ? 1 : m;
  }
}

__global__ void __launch_bounds__(256) join_pairs_ordered_kernel(const __grid_constant__ MatchParams p) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < p.n; r += stride) {
    const int32_t o = p.offs[r];
    const int m = walk_matches(p, r, [&](uint32_t b, int j) {
      p.out_p[o + j] = static_cast<int32_t>(r);
      p.out_b[o + j] = static_cast<int32_t>(b);
    });
    if (m == 0 && p.keep_unmatched) {
      p.out_p[o] = static_cast<int32_t>(r);
      p.out_b[o] = -1;
    }
  }
}

__global__ void flag_rows_kernel(const int32_t* __restrict__ v, int64_t n, int nonzero, int32_t* __restrict__ sel) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    sel[i] = (v[i] != 0) == (nonzero != 0) ? 1 : 0;
}

__global__ void flag_scatter_kernel(const int32_t* __restrict__ sel, const int32_t* __restrict__ pos, int64_t n,
                                    int32_t* __restrict__ rows) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    if (sel[i]) rows[pos[i]] = static_cast<int32_t>(i);
}

MatchParams match_params(const JoinTable& t, const TupleSet& probe, int probe_key) {
  const int64_t n = probe.num_rows();
  if (n >= INT32_MAX) fail(GFPDB_EUNSUPPORTED, "hash join probe batch must have fewer than 2^31 rows");
  const auto& pc = probe.column(probe_key);
  if (pc->type == DType::Utf8 || pc->type == DType::Float64)
    fail(GFPDB_EUNSUPPORTED, "hash join keys must be integer columns");
  const bool key32 = t.key_type != DType::Int64 && pc->type != DType::Int64;
  if (!key32 && t.key_type != DType::Int64) fail(GFPDB_EUNSUPPORTED, "int64 probe key against an int32 build key");
  const auto& bk = t.build->column(t.key_col);
  MatchParams p{};
  p.pkey = DevCol{pc->data, nullptr, static_cast<int32_t>(pc->type), 0};
  p.bkey = DevCol{bk->data, nullptr, static_cast<int32_t>(bk->type), 0};
  p.slots = t.slots->as<uint64_t>();
  p.mask = t.capacity - 1;
  p.key32 = key32 ? 1 : 0;
  p.n = n;
  return p;
}

}  // namespace

void join_match(const JoinTable& t, const TupleSet& probe, int probe_key, int32_t* counts, bool keep_unmatched,
                int32_t* matched, cudaStream_t s) {
  MatchParams p = match_params(t, probe, probe_key);
  p.counts = counts;
  p.keep_unmatched = keep_unmatched ? 1 : 0;
  p.matched = matched;
  if (p.n == 0) return;
  ProfScope prof("join_match_kernel", s);
  join_match_kernel<<<grid_for(p.n), 256, 0, s>>>(p);
  after_launch("join_match_kernel");
  prof.stop(static_cast<double>(p.n) * (dtype_width(probe.column(probe_key)->type) + (counts ? 4 : 0)));
}

void join_pairs_ordered(const JoinTable& t, const TupleSet& probe, int probe_key, bool keep_unmatched,
                        int32_t* matched, BufferPtr* pidx, BufferPtr* bidx, int64_t* n_out, cudaStream_t s) {
  const int64_t n = probe.num_rows();
  auto counts = make_buffer((n > 0 ? n : 1) * 4, s);
  auto offs = make_buffer((n + 1) * 4, s);
  join_match(t, probe, probe_key, counts->as<int32_t>(), keep_unmatched, matched, s);
  const int64_t total = n > 0 ? exclusive_scan_i32(counts->as<int32_t>(), offs->as<int32_t>(), n, s) : 0;
  *pidx = make_buffer((total > 0 ? total : 1) * 4, s);
  *bidx = make_buffer((total > 0 ? total : 1) * 4, s);
  *n_out = total;
  if (n == 0) return;
  MatchParams p = match_params(t, probe, probe_key);
  p.keep_unmatched = keep_unmatched ? 1 : 0;
  p.offs = offs->as<int32_t>();
  p.out_p = (*pidx)->as<int32_t>();
  p.out_b = (*bidx)->as<int32_t>();
  ProfScope prof("join_pairs_ordered_kernel", s);
  join_pairs_ordered_kernel<<<grid_for(n), 256, 0, s>>>(p);
  after_launch("join_pairs_ordered_kernel");
  prof.stop(static_cast<double>(n) * (dtype_width(probe.column(probe_key)->type) + 4) + static_cast<double>(total) * 8);
}

BufferPtr rows_where(const int32_t* v, int64_t n, bool nonzero, int64_t* n_out, cudaStream_t s) {
  *n_out = 0;
  if (n == 0) return make_buffer(4, s);
  auto sel = make_buffer(n * 4, s);
  auto pos = make_buffer((n + 1) * 4, s);
  flag_rows_kernel<<<grid_for(n), 256, 0, s>>>(v, n, nonzero ? 1 : 0, sel->as<int32_t>());
  after_launch("flag_rows_kernel");
  const int64_t total = exclusive_scan_i32(sel->as<int32_t>(), pos->as<int32_t>(), n, s);
  auto rows = make_buffer((total > 0 ? total : 1) * 4, s);
  if (total > 0) {
    flag_scatter_kernel<<<grid_for(n), 256, 0, s>>>(sel->as<int32_t>(), pos->as<int32_t>(), n, rows->as<int32_t>());
    after_launch("flag_scatter_kernel");
  }
  *n_out = total;
  return rows;
}

}  // namespace gfpdb
