// Bloom filter build: one thread per key, the key's block masks built in
// registers, then one atomicOr per non-zero word of the 256-bit block.
// Replaces ArrowBloomFilter::build / BlockedBloomFilter::Insert
// (fpdb-executor/src/physical/bloomfilter/ArrowBloomFilter.cpp:29-75;
// fpdb-tuple/src/arrow/exec/BloomFilter.cpp:110-137).
#include "bloom.cuh"
#include "launch.h"

namespace gfpdb {

namespace {

__global__ void __launch_bounds__(256)
    bloom_build_kernel(DevCol key, int64_t n, uint32_t* __restrict__ blocks, uint64_t num_blocks, int num_hashes) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
    const uint64_t h = hash_key(load_int(key, r));
    uint32_t m[8];
    bloom_masks(h, num_hashes, m);
    uint32_t* blk = blocks + static_cast<uint64_t>(bloom_block_of(h, num_blocks)) * 8;
#pragma unroll
    for (int w = 0; w < 8; ++w)
      if (m[w] != 0) atomicOr(blk + w, m[w]);
  }
}

}  // namespace

BloomPtr bloom_build(const std::vector<const Column*>& key_parts, int32_t bits_per_key, int32_t num_hashes,
                     cudaStream_t s) {
  if (bits_per_key < 1 || bits_per_key > 64) fail(GFPDB_EINVAL, "bits_per_key must be in [1, 64]");
  if (num_hashes < 1 || num_hashes > 4) fail(GFPDB_EINVAL, "num_hashes must be in [1, 4]");
  int64_t n = 0;
  for (auto* c : key_parts) {
    if (c->type != DType::Int32 && c->type != DType::Int64 && c->type != DType::Date32)
      fail(GFPDB_EUNSUPPORTED, "bloom filter keys must be int32, int64 or date32");
    n += c->length;
  }
  auto bf = std::make_shared<BloomFilterDev>();
  bf->num_keys = n;
  bf->num_hashes = num_hashes;
  bf->bits_per_key = bits_per_key;
  if (n > GFPDB_BLOOM_MAX_INPUT_SIZE) {
    // Too many keys: the filter is invalid and every probe passes.
    bf->valid = false;
    bf->num_blocks = 0;
    bf->blocks = make_buffer(32, s);
    return bf;
  }
  int64_t nb = (n * bits_per_key + 255) / 256;
  if (nb < 1) nb = 1;
  bf->num_blocks = nb;
  bf->blocks = make_buffer(nb * 32, s);
  GF_CUDA(cudaMemsetAsync(bf->blocks->data(), 0, nb * 32, s));
  for (auto* c : key_parts) {
    if (c->length == 0) continue;
    DevCol k{c->data, nullptr, static_cast<int32_t>(c->type), 0};
    int64_t blocks = (c->length + 255) / 256;
    int64_t cap = static_cast<int64_t>(num_sms()) * 8;
    ProfScope prof("bloom_build_kernel", s);
    bloom_build_kernel<<<static_cast<int>(blocks < cap ? blocks : cap), 256, 0, s>>>(
        k, c->length, bf->blocks->as<uint32_t>(), static_cast<uint64_t>(nb), num_hashes);
    after_launch("bloom_build_kernel");
    prof.stop(static_cast<double>(c->length) * dtype_width(c->type));
  }
  return bf;
}

}  // namespace gfpdb
