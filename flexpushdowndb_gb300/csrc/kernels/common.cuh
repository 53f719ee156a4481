// Device helpers shared by every kernel: status reporting, hashing, column
// loads, memory-ordered flags and the decoupled look-back used for
// single-pass stable compaction and prefix sums.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../host/runtime.h"
#include "../program.h"

namespace gfpdb {

constexpr uint64_t kEmptySlot = 0xFFFFFFFFFFFFFFFFull;

// Upper bound on any spin-wait on another CTA's flag. A CTA that waits this
// long records GFPDB_ETIMEDOUT in the call's status block and stops waiting,
// so a wait can never hang the device.
constexpr uint32_t kSpinLimit = 1u << 22;

__device__ __forceinline__ void raise_status(DevStatus* st, int32_t code, int32_t detail) {
  if (atomicCAS(&st->code, 0, code) == 0) st->detail = detail;
}

// 64-bit finaliser of MurmurHash3 (Austin Appleby, public domain): a
// bijective mix with full avalanche, used for bloom, join and group hashing.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

// Integer keys hash by value: an int32 key and an int64 key with the same
// value land in the same bucket, so join keys of mixed widths match.
__host__ __device__ __forceinline__ uint64_t hash_key(int64_t v) { return mix64(static_cast<uint64_t>(v) ^ 0x9e3779b97f4a7c15ull); }

// FNV-1a over bytes, then mixed: the hash of a utf8 value.
__device__ __forceinline__ uint64_t hash_bytes(const uint8_t* p, int32_t n) {
  uint64_t h = 0xcbf29ce484222325ull;
  for (int32_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 0x100000001b3ull;
  }
  return mix64(h ^ static_cast<uint64_t>(n));
}

__device__ __forceinline__ int64_t load_int(const DevCol& c, int64_t row) {
  if (c.type == CT_I64) return __ldg(static_cast<const long long*>(c.data) + row);
  return __ldg(static_cast<const int*>(c.data) + row);
}

// Hash of one row's key of n columns: integers by value (int32 and int64
// columns with equal values agree), utf8 by bytes, each column's hash folded
// in with a boost-style combine and a full mix. The composite join / bloom
// keys and the shuffle's slot assignment both use it.
constexpr uint64_t kRowKeySeed = 0x243f6a8885a308d3ull;
__device__ __forceinline__ uint64_t row_key_combine(uint64_t h, uint64_t v) {
  return mix64(h ^ (v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2)));
}
__device__ __forceinline__ uint64_t row_key_hash(const DevCol* cols, int n, int64_t row) {
  uint64_t h = kRowKeySeed;
  for (int c = 0; c < n; ++c) {
    const DevCol& col = cols[c];
    uint64_t v;
    if (col.type == CT_UTF8) {
      const int32_t b = col.offsets[row], e = col.offsets[row + 1];
      v = hash_bytes(static_cast<const uint8_t*>(col.data) + b, e - b);
    } else {
      v = hash_key(load_int(col, row));
    }
    h = row_key_combine(h, v);
  }
  return h;
}

__device__ __forceinline__ int64_t load_as_i64_bits(const DevCol& c, int64_t row) {
  if (c.type == CT_I64 || c.type == CT_F64) return __ldg(static_cast<const long long*>(c.data) + row);
  return __ldg(static_cast<const int*>(c.data) + row);
}

__device__ __forceinline__ uint64_t ld_acquire(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(uint64_t* p, uint64_t v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint32_t ld_acquire32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release32(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// ---- asynchronous bulk copies into shared memory (cp.async.bulk + mbarrier)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes mbarrier initialisation visible to the async proxy (bulk copies).
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Upper bound on polls of one mbarrier phase; each poll may suspend the
// thread for a bounded, hardware-defined time.
constexpr uint32_t kMbarSpinLimit = 1u << 20;

// Waits for the phase of `bar` with the given parity to complete; false if
// it did not within kMbarSpinLimit polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < kMbarSpinLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned)
// from global to this CTA's shared memory, completing on `bar`.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// Tile status words for decoupled look-back (Merrill & Garland, "Single-pass
// Parallel Prefix Scan with Decoupled Look-back", 2016): the top two bits
// say whether the word holds nothing yet, the tile's own aggregate, or the
// inclusive prefix through that tile.
constexpr uint64_t kFlagAgg = 1ull << 62;
constexpr uint64_t kFlagIncl = 2ull << 62;
constexpr uint64_t kValueMask = (1ull << 62) - 1;

// Called by all 32 lanes of one warp. Publishes `tile_total` for `tile` and
// returns the exclusive prefix (sum of all earlier tiles). Tiles must be
// handed out in increasing order (atomic ticket) so that every earlier tile
// belongs to a CTA that is already running; each wait is still bounded.
__device__ __forceinline__ uint64_t lookback_exclusive(uint64_t* status, int64_t tile, uint64_t tile_total,
                                                       DevStatus* st) {
  const int lane = threadIdx.x & 31;
  if (tile == 0) {
    if (lane == 0) st_release(&status[0], kFlagIncl | tile_total);
    return 0;
  }
  if (lane == 0) st_release(&status[tile], kFlagAgg | tile_total);
  uint64_t excl = 0;
  int64_t window = tile - 1;
  for (;;) {
    const int64_t j = window - lane;
    uint64_t v;
    uint32_t spins = 0;
    for (;;) {
      v = j >= 0 ? ld_acquire(&status[j]) : kFlagIncl;
      const bool missing = (v & ~kValueMask) == 0;
      if (!__any_sync(0xffffffffu, missing)) break;
      if (++spins > kSpinLimit) {
        if (lane == 0) raise_status(st, GFPDB_ETIMEDOUT, 1);
        v = kFlagIncl;  // give up: the call reports the timeout
        break;
      }
      __nanosleep(64);
    }
    const uint32_t incl = __ballot_sync(0xffffffffu, (v & ~kValueMask) == kFlagIncl);
    uint64_t mine = v & kValueMask;
    if (incl != 0) {
      const int first = __ffs(incl) - 1;
      if (lane > first) mine = 0;
    }
    for (int d = 16; d > 0; d >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, d);
    excl += __shfl_sync(0xffffffffu, mine, 0);
    if (incl != 0) break;
    window -= 32;
  }
  if (lane == 0) st_release(&status[tile], kFlagIncl | (excl + tile_total));
  return excl;
}

// Block-wide exclusive sum of one int per thread (blockDim.x <= 1024).
// Returns the thread's exclusive prefix; *total gets the block sum.
template <int THREADS>
__device__ __forceinline__ int block_exclusive_sum(int x, int* total, int* s_warp) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  constexpr int NW = THREADS / 32;
  int incl = x;
  for (int d = 1; d < 32; d <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = lane < NW ? s_warp[lane] : 0;
    int wi = w;
    for (int d = 1; d < 32; d <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, wi, d);
      if (lane >= d) wi += y;
    }
    if (lane < NW) s_warp[lane] = wi - w;
    if (lane == NW - 1) s_warp[NW] = wi;
  }
  __syncthreads();
  int r = incl - x + s_warp[warp];
  *total = s_warp[NW];
  return r;
}

// Barrier over the first THREADS threads of the block only (named barrier
// BAR_ID), for warp-specialised kernels whose other warps never join.
template <int BAR_ID, int THREADS>
__device__ __forceinline__ void named_sync() {
  asm volatile("bar.sync %0, %1;" ::"n"(BAR_ID), "n"(THREADS) : "memory");
}

// block_exclusive_sum over threads [0, THREADS) synchronised by named
// barrier BAR_ID.
template <int BAR_ID, int THREADS>
__device__ __forceinline__ int named_exclusive_sum(int x, int* total, int* s_warp) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  constexpr int NW = THREADS / 32;
  int incl = x;
  for (int d = 1; d < 32; d <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  named_sync<BAR_ID, THREADS>();
  if (warp == 0) {
    int w = lane < NW ? s_warp[lane] : 0;
    int wi = w;
    for (int d = 1; d < 32; d <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, wi, d);
      if (lane >= d) wi += y;
    }
    if (lane < NW) s_warp[lane] = wi - w;
    if (lane == NW - 1) s_warp[NW] = wi;
  }
  named_sync<BAR_ID, THREADS>();
  int r = incl - x + s_warp[warp];
  *total = s_warp[NW];
  return r;
}

}  // namespace gfpdb
