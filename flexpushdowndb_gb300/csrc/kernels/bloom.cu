// Bloom filter build: one thread per key, the key's block masks built in
// registers, then one atomicOr per non-zero word of the 256-bit block.
// Replaces ArrowBloomFilter::build / BlockedBloomFilter::Insert
// (fpdb-executor/src/physical/bloomfilter/ArrowBloomFilter.cpp:29-75;
// fpdb-tuple/src/arrow/exec/BloomFilter.cpp:110-137).
//
// When the key columns come from deferred TupleSets (row counts known only
// on the device), the filter is allocated for the upper bound and a one-thread
// kernel sizes it from the device counts (same formula as the host path), so
// the filter is bit-identical to one built from exact inputs.
#include "bloom.cuh"
#include "launch.h"

namespace gfpdb {

namespace {

struct BloomHeader {
  uint64_t num_blocks;
  int32_t valid;
  int32_t pad;
  int64_t num_keys;
};

constexpr int kMaxBloomParts = 256;

struct BloomSizeParams {
  const int64_t* n_dev[kMaxBloomParts];
  int64_t cap[kMaxBloomParts];
  int32_t n_parts;
  int32_t bits_per_key;
  BloomHeader* hdr;
};

// Filter size from the device key counts (same formula as the host path);
// every thread of every build launch computes it, and the first thread of the
// first launch records it in the header for the probes.
__device__ __forceinline__ void bloom_size(const BloomSizeParams& p, uint64_t* nb, bool* valid) {
  int64_t total = 0;
  for (int i = 0; i < p.n_parts; ++i) total += clamp_rows(p.n_dev[i], p.cap[i]);
  int64_t blocks = (total * p.bits_per_key + 255) / 256;
  if (blocks < 1) blocks = 1;
  *nb = static_cast<uint64_t>(blocks);
  *valid = total <= GFPDB_BLOOM_MAX_INPUT_SIZE;
  if (p.hdr != nullptr && blockIdx.x == 0 && threadIdx.x == 0 && p.n_parts >= 0) {
    p.hdr->num_keys = total;
    p.hdr->valid = *valid ? 1 : 0;
    p.hdr->num_blocks = *nb;
  }
}

__global__ void __launch_bounds__(256)
    bloom_build_kernel(DevCol key, int64_t cap, const int64_t* n_dev, uint32_t* __restrict__ blocks,
                       uint64_t num_blocks, const __grid_constant__ BloomSizeParams sp, int num_hashes) {
  const int64_t n = clamp_rows(n_dev, cap);
  uint64_t nb = num_blocks;
  if (sp.hdr != nullptr) {
    bool valid = true;
    bloom_size(sp, &nb, &valid);
    if (!valid) return;
  }
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
    const uint64_t h = bloom_hash(load_int(key, r));
    uint32_t m[8];
    bloom_masks(h, num_hashes, m);
    uint32_t* blk = blocks + static_cast<uint64_t>(bloom_block_of(h, nb)) * 8;
#pragma unroll
    for (int w = 0; w < 8; ++w)
      if (m[w] != 0) atomicOr(blk + w, m[w]);
  }
}

// Several filters over the same rows, each on its own key column, built in
// one pass: a thread loads each filter's key of its row and sets that
// filter's bits. A filter sized on the device (hdr set) takes its size from
// the shared part counts with its own bits per key, as bloom_size does.
struct BloomMultiParams {
  DevCol key[kBloomBuildManyMax];
  uint32_t* blocks[kBloomBuildManyMax];
  uint64_t num_blocks[kBloomBuildManyMax];  // exact size, or the capacity when hdr is set
  BloomHeader* hdr[kBloomBuildManyMax];
  int32_t num_hashes[kBloomBuildManyMax];
  int32_t bits_per_key[kBloomBuildManyMax];
  int32_t n;
};

__global__ void __launch_bounds__(256)
    bloom_build_many_kernel(int64_t cap, const int64_t* n_dev, const __grid_constant__ BloomMultiParams p,
                            const __grid_constant__ BloomSizeParams sp) {
  const int64_t n = clamp_rows(n_dev, cap);
  int64_t total = -1;  // keys over every part, for the filters sized on the device
  uint64_t nb[kBloomBuildManyMax];
  bool live[kBloomBuildManyMax];
#pragma unroll
  for (int f = 0; f < kBloomBuildManyMax; ++f) {
    nb[f] = f < p.n ? p.num_blocks[f] : 1;
    live[f] = f < p.n;
    if (f < p.n && p.hdr[f] != nullptr) {
      if (total < 0) {
        total = 0;
        for (int i = 0; i < sp.n_parts; ++i) total += clamp_rows(sp.n_dev[i], sp.cap[i]);
      }
      int64_t blocks = (total * p.bits_per_key[f] + 255) / 256;
      if (blocks < 1) blocks = 1;
      nb[f] = static_cast<uint64_t>(blocks);
      live[f] = total <= GFPDB_BLOOM_MAX_INPUT_SIZE;
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        p.hdr[f]->num_keys = total;
        p.hdr[f]->valid = live[f] ? 1 : 0;
        p.hdr[f]->num_blocks = nb[f];
      }
    }
  }
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
    // every filter's key first, so the loads are in flight together (the
    // bit updates below could alias them as far as the compiler knows)
    int64_t key[kBloomBuildManyMax];
#pragma unroll
    for (int f = 0; f < kBloomBuildManyMax; ++f) key[f] = live[f] ? load_int(p.key[f], r) : 0;
#pragma unroll
    for (int f = 0; f < kBloomBuildManyMax; ++f) {
      if (!live[f]) continue;
      const uint64_t h = bloom_hash(key[f]);
      uint32_t* blk = p.blocks[f] + static_cast<uint64_t>(bloom_block_of(h, nb[f])) * 8;
      // one bit per hash (at most four): the same bits bloom_masks sets
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (i < p.num_hashes[f]) {
          const uint32_t b = static_cast<uint32_t>(h >> (8 * i)) & 0xFFu;
          atomicOr(blk + (b >> 5), 1u << (b & 31));
        }
    }
  }
}

// A filter's shell over up to n keys: sized for them (for at most
// GFPDB_BLOOM_MAX_INPUT_SIZE when the count is a device-side upper bound),
// or invalid when more are known on the host; zeroed blocks, and a header
// for a filter sized on the device.
std::shared_ptr<BloomFilterDev> bloom_alloc(int64_t n, int32_t bits_per_key, int32_t num_hashes, bool deferred,
                                            cudaStream_t s) {
  if (bits_per_key < 1 || bits_per_key > 64) fail(GFPDB_EINVAL, "bits_per_key must be in [1, 64]");
  if (num_hashes < 1 || num_hashes > 4) fail(GFPDB_EINVAL, "num_hashes must be in [1, 4]");
  auto bf = std::make_shared<BloomFilterDev>();
  bf->num_keys = n;
  bf->num_hashes = num_hashes;
  bf->bits_per_key = bits_per_key;
  if (!deferred && n > GFPDB_BLOOM_MAX_INPUT_SIZE) {
    bf->valid = false;
    bf->num_blocks = 0;
    bf->blocks = make_buffer(32, s);
    return bf;
  }
  const int64_t n_alloc = n < GFPDB_BLOOM_MAX_INPUT_SIZE ? n : GFPDB_BLOOM_MAX_INPUT_SIZE;
  int64_t nb = (n_alloc * bits_per_key + 255) / 256;
  if (nb < 1) nb = 1;
  bf->num_blocks = nb;
  bf->blocks = make_filled(nb * 32, 0, s);
  if (deferred) {
    bf->header = make_buffer(sizeof(BloomHeader), s);
    BloomHeader* hdr = bf->header->as<BloomHeader>();
    bf->nblocks_dev = &hdr->num_blocks;
    bf->valid_dev = &hdr->valid;
  }
  return bf;
}

}  // namespace

std::vector<BloomPtr> bloom_build_many(const std::vector<std::vector<const Column*>>& key_parts,
                                       const std::vector<int32_t>& bits_per_key, const std::vector<int32_t>& num_hashes,
                                       cudaStream_t s, const std::vector<const int64_t*>& part_rows_dev) {
  const size_t nf = key_parts.size();
  if (nf == 0 || nf > static_cast<size_t>(kBloomBuildManyMax) || bits_per_key.size() != nf || num_hashes.size() != nf)
    fail(GFPDB_EINVAL, "bloom_build_many: 1 to 8 filters, each with its bits per key and hash count");
  const size_t np = key_parts[0].size();
  bool deferred = false;
  for (auto* d : part_rows_dev) deferred |= d != nullptr;
  if (deferred && np > static_cast<size_t>(kMaxBloomParts)) fail(GFPDB_EUNSUPPORTED, "too many deferred bloom inputs");
  int64_t n = 0;
  for (size_t i = 0; i < np; ++i) {
    for (size_t f = 0; f < nf; ++f) {
      if (key_parts[f].size() != np || key_parts[f][i]->length != key_parts[0][i]->length)
        fail(GFPDB_EINVAL, "bloom_build_many: every filter's key parts are the same rows");
      const DType t = key_parts[f][i]->type;
      if (t != DType::Int32 && t != DType::Int64 && t != DType::Date32)
        fail(GFPDB_EUNSUPPORTED, "bloom filter keys must be int32, int64 or date32");
    }
    n += key_parts[0][i]->length;
  }
  std::vector<std::shared_ptr<BloomFilterDev>> filters;
  BloomMultiParams mp{};
  std::vector<int> slot_of(nf, -1);  // kernel slot of each filter (none for an invalid one)
  for (size_t f = 0; f < nf; ++f) {
    filters.push_back(bloom_alloc(n, bits_per_key[f], num_hashes[f], deferred, s));
    const auto& bf = filters.back();
    if (!bf->valid) continue;
    slot_of[f] = mp.n;
    mp.blocks[mp.n] = bf->blocks->as<uint32_t>();
    mp.num_blocks[mp.n] = static_cast<uint64_t>(bf->num_blocks);
    mp.hdr[mp.n] = deferred ? bf->header->as<BloomHeader>() : nullptr;
    mp.num_hashes[mp.n] = num_hashes[f];
    mp.bits_per_key[mp.n] = bits_per_key[f];
    ++mp.n;
  }
  if (mp.n > 0) {
    BloomSizeParams sp{};
    if (deferred) {
      sp.n_parts = static_cast<int32_t>(np);
      for (size_t i = 0; i < np; ++i) {
        sp.n_dev[i] = i < part_rows_dev.size() ? part_rows_dev[i] : nullptr;
        sp.cap[i] = key_parts[0][i]->length;
      }
    }
    bool header_written = !deferred;
    for (size_t i = 0; i < np; ++i) {
      const int64_t len = key_parts[0][i]->length;
      // the first launch of device-sized filters writes their headers, so it
      // runs even for an empty part
      if (len == 0 && header_written) continue;
      header_written = true;
      for (size_t f = 0; f < nf; ++f)
        if (slot_of[f] >= 0)
          mp.key[slot_of[f]] = DevCol{key_parts[f][i]->data, nullptr, static_cast<int32_t>(key_parts[f][i]->type), 0};
      const int64_t* n_dev = i < part_rows_dev.size() ? part_rows_dev[i] : nullptr;
      int64_t blocks = (len + 255) / 256;
      const int64_t cap = static_cast<int64_t>(num_sms()) * 4;
      if (blocks < 1) blocks = 1;
      ProfScope prof("bloom_build_many_kernel", s);
      bloom_build_many_kernel<<<static_cast<int>(blocks < cap ? blocks : cap), 256, 0, s>>>(len, n_dev, mp, sp);
      after_launch("bloom_build_many_kernel");
      double bytes = 0;
      for (size_t f = 0; f < nf; ++f) bytes += static_cast<double>(len) * dtype_width(key_parts[f][i]->type);
      prof.stop(bytes);
    }
  }
  return std::vector<BloomPtr>(filters.begin(), filters.end());
}

BloomPtr bloom_build(const std::vector<const Column*>& key_parts, int32_t bits_per_key, int32_t num_hashes,
                     cudaStream_t s, const std::vector<const int64_t*>& part_rows_dev) {
  if (bits_per_key < 1 || bits_per_key > 64) fail(GFPDB_EINVAL, "bits_per_key must be in [1, 64]");
  if (num_hashes < 1 || num_hashes > 4) fail(GFPDB_EINVAL, "num_hashes must be in [1, 4]");
  bool deferred = false;
  for (auto* d : part_rows_dev) deferred |= d != nullptr;
  int64_t n = 0;  // exact key count, or its upper bound when deferred
  for (auto* c : key_parts) {
    if (c->type != DType::Int32 && c->type != DType::Int64 && c->type != DType::Date32)
      fail(GFPDB_EUNSUPPORTED, "bloom filter keys must be int32, int64 or date32");
    n += c->length;
  }
  auto bf = std::make_shared<BloomFilterDev>();
  bf->num_keys = n;
  bf->num_hashes = num_hashes;
  bf->bits_per_key = bits_per_key;
  if (!deferred && n > GFPDB_BLOOM_MAX_INPUT_SIZE) {
    // Too many keys: the filter is invalid and every probe passes.
    bf->valid = false;
    bf->num_blocks = 0;
    bf->blocks = make_buffer(32, s);
    return bf;
  }
  const int64_t n_alloc = n < GFPDB_BLOOM_MAX_INPUT_SIZE ? n : GFPDB_BLOOM_MAX_INPUT_SIZE;
  int64_t nb = (n_alloc * bits_per_key + 255) / 256;
  if (nb < 1) nb = 1;
  bf->num_blocks = nb;  // exact size, or the capacity of a device-sized filter
  bf->blocks = make_filled(nb * 32, 0, s);
  BloomSizeParams sp{};
  if (deferred) {
    if (key_parts.size() > static_cast<size_t>(kMaxBloomParts))
      fail(GFPDB_EUNSUPPORTED, "too many deferred bloom inputs");
    bf->header = make_buffer(sizeof(BloomHeader), s);
    BloomHeader* hdr = bf->header->as<BloomHeader>();
    sp.n_parts = static_cast<int32_t>(key_parts.size());
    sp.bits_per_key = bits_per_key;
    sp.hdr = hdr;
    for (size_t i = 0; i < key_parts.size(); ++i) {
      sp.n_dev[i] = i < part_rows_dev.size() ? part_rows_dev[i] : nullptr;
      sp.cap[i] = key_parts[i]->length;
    }
    bf->nblocks_dev = &hdr->num_blocks;
    bf->valid_dev = &hdr->valid;
  }
  bool header_written = !deferred;
  for (size_t i = 0; i < key_parts.size(); ++i) {
    const Column* c = key_parts[i];
    // The first launch of a device-sized filter also writes its header, so
    // it runs even for an empty part.
    if (c->length == 0 && header_written) continue;
    header_written = true;
    DevCol k{c->data, nullptr, static_cast<int32_t>(c->type), 0};
    const int64_t* n_dev = i < part_rows_dev.size() ? part_rows_dev[i] : nullptr;
    int64_t blocks = (c->length + 255) / 256;
    int64_t cap = static_cast<int64_t>(num_sms()) * 4;  // grid-stride: four CTAs per SM keep the atomics busy
    ProfScope prof("bloom_build_kernel", s);
    if (blocks < 1) blocks = 1;
    bloom_build_kernel<<<static_cast<int>(blocks < cap ? blocks : cap), 256, 0, s>>>(
        k, c->length, n_dev, bf->blocks->as<uint32_t>(), static_cast<uint64_t>(nb), sp, num_hashes);
    after_launch("bloom_build_kernel");
    prof.stop(static_cast<double>(c->length) * dtype_width(c->type));
  }
  return bf;
}

}  // namespace gfpdb
