// Blocked bloom filter layout shared by the build kernel and the fused probe.
//
// A filter is num_blocks blocks of 256 bits (8 x uint32, one 32-byte DRAM
// sector). A key's 64-bit hash (bloom_hash: one multiply by 2^64 / phi,
// Fibonacci hashing, and an xorshift that folds the well-mixed high bits
// into the low ones; as few false positives as the MurmurHash3 finaliser on
// sequential, strided and random keys, at a third of its instructions)
// picks its block from the high 32 bits
// (multiply-shift range reduction) and `num_hashes` bit positions inside
// the block from consecutive bytes of the low 32 bits (byte b: word b >> 5,
// bit b & 31). A probe therefore touches one sector, and a build sets its
// bits with at most num_hashes atomicOr operations on that sector.
//
// This replaces the reference's vendored Arrow blocked filter (57-bit masks
// in 64-bit blocks, fpdb-tuple/include/fpdb/tuple/arrow/exec/BloomFilter.h:41-268)
// and the Carter-Wegman flat filter (fpdb-executor/src/physical/bloomfilter/BloomFilter.cpp:55-257).
// Only "no false negatives" matters for query results: joins after the
// bloom remove every false positive.
#pragma once

#include "common.cuh"

namespace gfpdb {

__host__ __device__ __forceinline__ uint64_t bloom_hash(int64_t k) {
  const uint64_t h = static_cast<uint64_t>(k) * 0x9E3779B97F4A7C15ull;
  return h ^ (h >> 29);
}

__host__ __device__ __forceinline__ uint32_t bloom_block_of(uint64_t h, uint64_t num_blocks) {
  return static_cast<uint32_t>(((h >> 32) * num_blocks) >> 32);
}

// Word masks of the key inside its block: returns the 8 per-word masks.
__host__ __device__ __forceinline__ void bloom_masks(uint64_t h, int num_hashes, uint32_t m[8]) {
  for (int w = 0; w < 8; ++w) m[w] = 0;
  for (int i = 0; i < num_hashes; ++i) {
    const uint32_t b = static_cast<uint32_t>(h >> (8 * i)) & 0xFFu;
    m[b >> 5] |= 1u << (b & 31);
  }
}

__device__ __forceinline__ bool bloom_test(const uint32_t* blk, uint64_t h, int num_hashes) {
  bool ok = true;
  for (int i = 0; i < num_hashes; ++i) {
    const uint32_t b = static_cast<uint32_t>(h >> (8 * i)) & 0xFFu;
    ok &= (blk[b >> 5] >> (b & 31)) & 1u;
  }
  return ok;
}

}  // namespace gfpdb
