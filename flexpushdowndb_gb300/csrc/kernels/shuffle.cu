// Hash partitioning of a TupleSet's rows into slots: the GPU form of
// ShuffleKernel2::shuffle (fpdb-executor/src/physical/shuffle/ShuffleKernel2.cpp:28-125),
// which hashes the shuffle columns of every row (RecordBatchHasher), appends
// the row id to the list of slot hash % numSlots, takes the rows in slot order
// and slices the result into one TupleSet per slot. Rows keep their input
// order within a slot.
//
// Here the slot of a row is a fast range of a 64-bit mix of the row's key
// hash (row_key_hash: integers by value, utf8 by bytes), independent of the
// low bits that join and group tables index by and of the bloom's block bits.
// The reference's partition function is Arrow's HashMultiColumn; which slot a
// key lands in does not change any query's result, only that equal keys land
// in the same slot.
//
// Three launches, all stable and without global atomics, over tiles of
// 512 rows per warp of a block (4096 rows for 8 warps):
//   shuffle_count_kernel   the slots of a tile's rows (several key loads in
//                          flight per thread), counted by shared-memory
//                          atomics; the counts land slot-major in a
//                          [slots][tiles] matrix;
//   scan_i32_kernel        one exclusive prefix sum over the matrix gives each
//                          (slot, tile) its first output row;
//   shuffle_scatter_kernel the tile's rows ranked in shared memory (a lane's
//                          peers with the same slot from one ballot per slot
//                          bit): per-warp counts of each slot, scanned across warps and
//                          slots, give every row its place in the tile's
//                          slot order (input order kept); then each column
//                          leaves in that order, consecutive threads writing
//                          consecutive rows of one slot's run, so the writes
//                          are whole sectors rather than one value per
//                          sector. utf8 columns are gathered afterwards
//                          through the inverse permutation the same kernel
//                          writes.
#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "launch.h"

namespace gfpdb {
namespace {

constexpr int kShufMaxFixed = 24;   // fixed-width columns scattered per launch
constexpr int kShufRowsPerWarp = 512;
constexpr int kShufUnroll = 4;      // key loads in flight per thread

struct ShufKeys {
  DevCol keys[kMaxKeyColumns];
  int32_t n_keys;
  uint32_t slots;
  int64_t n;       // rows
  int32_t tile;    // rows per block: warps * kShufRowsPerWarp
  int32_t slot_bits;  // bits of a slot number (0 for one slot)
  int64_t ntiles;
};

struct ShufScatter {
  const void* src[kShufMaxFixed];
  void* dst[kShufMaxFixed];
  int8_t width[kShufMaxFixed];
  int32_t n_fixed;
  int32_t pad;
  const int32_t* starts;  // scanned counts, [slots][ntiles]
  int32_t* inverse;       // inverse[out row] = input row (utf8 columns), or null
};

__device__ __forceinline__ uint32_t slot_of(uint64_t h, uint32_t slots) {
  const uint64_t g = mix64(h ^ 0x5851f42d4c957f2dull);
  return static_cast<uint32_t>(((g >> 32) * slots) >> 32);
}

// Slots of rows [begin, begin + rows) into out[0, rows): each thread takes
// rows tid, tid + blockDim, ..., kShufUnroll of them per round.
__device__ __forceinline__ void tile_slots(const ShufKeys& p, int64_t begin, int rows, uint16_t* out) {
  if (p.n_keys == 1 && p.keys[0].type != CT_UTF8) {  // one integer key: the loads first, then the hashes
    for (int base = 0; base < rows; base += kShufUnroll * blockDim.x) {
      int64_t v[kShufUnroll];
#pragma unroll
      for (int u = 0; u < kShufUnroll; ++u) {
        const int i = base + u * blockDim.x + threadIdx.x;
        v[u] = i < rows ? load_int(p.keys[0], begin + i) : 0;
      }
#pragma unroll
      for (int u = 0; u < kShufUnroll; ++u) {
        const int i = base + u * blockDim.x + threadIdx.x;
        if (i < rows) out[i] = static_cast<uint16_t>(slot_of(row_key_combine(kRowKeySeed, hash_key(v[u])), p.slots));
      }
    }
    return;
  }
  for (int base = 0; base < rows; base += kShufUnroll * blockDim.x) {
    uint64_t h[kShufUnroll];
#pragma unroll
    for (int u = 0; u < kShufUnroll; ++u) {
      const int i = base + u * blockDim.x + threadIdx.x;
      h[u] = i < rows ? row_key_hash(p.keys, p.n_keys, begin + i) : 0;
    }
#pragma unroll
    for (int u = 0; u < kShufUnroll; ++u) {
      const int i = base + u * blockDim.x + threadIdx.x;
      if (i < rows) out[i] = static_cast<uint16_t>(slot_of(h[u], p.slots));
    }
  }
}

// Lanes of the warp whose slot equals this lane's (the lane itself
// included), from one ballot per slot bit: the live lanes agreeing with this
// lane on every bit.
__device__ __forceinline__ unsigned slot_peers(uint32_t s, bool live, int bits) {
  unsigned peers = __ballot_sync(0xffffffffu, live);
  for (int b = 0; b < bits; ++b) {
    const unsigned ones = __ballot_sync(0xffffffffu, (s >> b) & 1u);
    peers &= ((s >> b) & 1u) ? ones : ~ones;
  }
  return peers;
}

__global__ void __launch_bounds__(256) shuffle_count_kernel(const __grid_constant__ ShufKeys p, int32_t* counts) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  int32_t* hist = reinterpret_cast<int32_t*>(s_raw);
  const int64_t begin = static_cast<int64_t>(blockIdx.x) * p.tile;
  const int rows = static_cast<int>(begin + p.tile < p.n ? p.tile : p.n - begin);
  for (uint32_t i = threadIdx.x; i < p.slots; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  const bool one_int_key = p.n_keys == 1 && p.keys[0].type != CT_UTF8;
  for (int base = 0; base < rows; base += kShufUnroll * blockDim.x) {
    uint64_t h[kShufUnroll];
    if (one_int_key) {
      int64_t v[kShufUnroll];
#pragma unroll
      for (int u = 0; u < kShufUnroll; ++u) {
        const int i = base + u * blockDim.x + threadIdx.x;
        v[u] = i < rows ? load_int(p.keys[0], begin + i) : 0;
      }
#pragma unroll
      for (int u = 0; u < kShufUnroll; ++u) h[u] = row_key_combine(kRowKeySeed, hash_key(v[u]));
    } else {
#pragma unroll
      for (int u = 0; u < kShufUnroll; ++u) {
        const int i = base + u * blockDim.x + threadIdx.x;
        h[u] = i < rows ? row_key_hash(p.keys, p.n_keys, begin + i) : 0;
      }
    }
#pragma unroll
    for (int u = 0; u < kShufUnroll; ++u)
      if (base + u * static_cast<int>(blockDim.x) + static_cast<int>(threadIdx.x) < rows)
        atomicAdd(&hist[slot_of(h[u], p.slots)], 1);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < p.slots; i += blockDim.x)
    counts[static_cast<int64_t>(i) * p.ntiles + blockIdx.x] = hist[i];
}

// Exclusive prefix sum of v[0, n) in shared memory by the whole block.
__device__ __forceinline__ void block_exclusive_scan(int32_t* v, int n, int32_t* warp_sums) {
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int lo = threadIdx.x * per;
  const int hi = lo + per < n ? lo + per : n;
  int32_t sum = 0;
  for (int k = lo; k < hi; ++k) sum += v[k];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t incl = sum;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int32_t t = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += t;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    int32_t run = 0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) {
      const int32_t t = warp_sums[w];
      warp_sums[w] = run;
      run += t;
    }
  }
  __syncthreads();
  int32_t excl = warp_sums[warp] + incl - sum;
  for (int k = lo; k < hi; ++k) {
    const int32_t t = v[k];
    v[k] = excl;
    excl += t;
  }
}

__global__ void __launch_bounds__(256) shuffle_scatter_kernel(const __grid_constant__ ShufKeys p,
                                                              const __grid_constant__ ShufScatter q) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  __shared__ int32_t warp_sums[32];
  const int tile = p.tile;
  const int nw = blockDim.x >> 5;
  const uint32_t slots = p.slots;
  int32_t* sdest = reinterpret_cast<int32_t*>(s_raw);  // [tile] output row of the tile's i-th row in slot order
  int32_t* tbase = sdest + tile;                         // [slots] first position of a slot in the tile's order
  int32_t* tstart = tbase + slots;                       // [slots] the slot's first output row for this tile
  uint16_t* srow = reinterpret_cast<uint16_t*>(tstart + slots);  // [tile] tile row at each position
  uint16_t* sslot = srow + tile;                                  // [tile] slot of each tile row
  uint16_t* wcnt = sslot + tile;                                  // [warps][slots]
  const int64_t begin = static_cast<int64_t>(blockIdx.x) * tile;
  const int rows = static_cast<int>(begin + tile < p.n ? tile : p.n - begin);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  for (uint32_t i = threadIdx.x; i < nw * slots; i += blockDim.x) wcnt[i] = 0;
  for (uint32_t i = threadIdx.x; i < slots; i += blockDim.x)
    tstart[i] = q.starts[static_cast<int64_t>(i) * p.ntiles + blockIdx.x];
  tile_slots(p, begin, rows, sslot);
  __syncthreads();

  // Per-warp counts over the warp's rows [warp * R, (warp + 1) * R).
  const int r0 = warp * kShufRowsPerWarp;
  uint16_t* mine = wcnt + static_cast<int64_t>(warp) * slots;
  for (int j = r0; j < r0 + kShufRowsPerWarp; j += 32) {
    const int i = j + lane;
    const bool live = i < rows;
    const uint32_t s = live ? sslot[i] : 0u;
    const unsigned peers = slot_peers(s, live, p.slot_bits);
    if (live && lane == __ffs(peers) - 1) mine[s] = static_cast<uint16_t>(mine[s] + __popc(peers));
    __syncwarp();
  }
  __syncthreads();
  // Exclusive across warps per slot (in place), the tile's count per slot.
  for (uint32_t s = threadIdx.x; s < slots; s += blockDim.x) {
    int32_t run = 0;
    for (int w = 0; w < nw; ++w) {
      const int32_t c = wcnt[static_cast<int64_t>(w) * slots + s];
      wcnt[static_cast<int64_t>(w) * slots + s] = static_cast<uint16_t>(run);
      run += c;
    }
    tbase[s] = run;
  }
  __syncthreads();
  block_exclusive_scan(tbase, static_cast<int>(slots), warp_sums);
  __syncthreads();

  // Each row's position in the tile's slot order, and its output row.
  const unsigned below = (1u << lane) - 1u;
  for (int j = r0; j < r0 + kShufRowsPerWarp; j += 32) {
    const int i = j + lane;
    const bool live = i < rows;
    const uint32_t s = live ? sslot[i] : 0u;
    const unsigned peers = slot_peers(s, live, p.slot_bits);
    if (live) {
      const int32_t within = mine[s] + __popc(peers & below);
      const int32_t lp = tbase[s] + within;
      srow[lp] = static_cast<uint16_t>(i);
      sdest[lp] = tstart[s] + within;
    }
    __syncwarp();
    if (live && lane == __ffs(peers) - 1) mine[s] = static_cast<uint16_t>(mine[s] + __popc(peers));
    __syncwarp();
  }
  __syncthreads();

  // The columns, in the tile's slot order.
  for (int c = 0; c < q.n_fixed; ++c) {
    if (q.width[c] == 8) {
      const long long* src = static_cast<const long long*>(q.src[c]) + begin;
      int64_t* dst = static_cast<int64_t*>(q.dst[c]);
      for (int i = threadIdx.x; i < rows; i += blockDim.x) dst[sdest[i]] = __ldg(src + srow[i]);
    } else {
      const int* src = static_cast<const int*>(q.src[c]) + begin;
      int32_t* dst = static_cast<int32_t*>(q.dst[c]);
      for (int i = threadIdx.x; i < rows; i += blockDim.x) dst[sdest[i]] = __ldg(src + srow[i]);
    }
  }
  if (q.inverse != nullptr)
    for (int i = threadIdx.x; i < rows; i += blockDim.x)
      q.inverse[sdest[i]] = static_cast<int32_t>(begin + srow[i]);
}

}  // namespace

ShuffleResult shuffle_rows(const TupleSetPtr& in_ts, const std::vector<std::string>& keys, int64_t num_slots,
                           cudaStream_t s) {
  if (keys.empty() || keys.size() > static_cast<size_t>(kMaxKeyColumns))
    fail(GFPDB_EINVAL, "a shuffle key has 1 to 8 columns");
  if (num_slots < 1 || num_slots > kShuffleMaxSlots)
    fail(GFPDB_EINVAL, "shuffle slots must be 1 to " + std::to_string(kShuffleMaxSlots));
  TupleSetPtr in = resolved(in_ts, s);
  const int64_t n = in->num_rows();
  if (n > INT32_MAX) fail(GFPDB_EUNSUPPORTED, "a shuffle input has at most 2^31 - 1 rows");

  ShufKeys p;
  std::memset(&p, 0, sizeof(p));
  for (size_t i = 0; i < keys.size(); ++i) {
    const auto& c = in->column(in->require_column(keys[i]));
    if (c->type == DType::Float64) fail(GFPDB_EUNSUPPORTED, "float64 shuffle column '" + keys[i] + "'");
    p.keys[i] = DevCol{c->data, c->offsets, static_cast<int32_t>(c->type), 0};
  }
  p.n_keys = static_cast<int32_t>(keys.size());
  p.slots = static_cast<uint32_t>(num_slots);
  p.n = n;

  ShuffleResult r;
  r.offsets.assign(num_slots + 1, 0);
  r.offsets[num_slots] = n;
  if (n == 0) {
    r.rows = in;
    return r;
  }

  // Tiles of 8 warps x 512 rows; the [slots][tiles] count matrix then holds
  // at most a quarter as many cells as rows (slots <= 1024).
  constexpr int kWarps = 8;
  p.tile = kWarps * kShufRowsPerWarp;
  p.ntiles = (n + p.tile - 1) / p.tile;
  const int blocks = static_cast<int>(p.ntiles);
  p.slot_bits = num_slots > 1 ? 64 - __builtin_clzll(static_cast<unsigned long long>(num_slots - 1)) : 0;
  const int64_t smem_count = num_slots * 4;
  const int64_t smem_scatter = static_cast<int64_t>(p.tile) * 4 + num_slots * 8 + static_cast<int64_t>(p.tile) * 4 +
                               kWarps * num_slots * 2;
  if (smem_scatter > 48 * 1024)
    GF_CUDA(cudaFuncSetAttribute(shuffle_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(smem_scatter)));

  const int64_t cells = num_slots * p.ntiles;
  auto counts = make_buffer(cells * 4, s);
  auto starts = make_buffer((cells + 1) * 4, s);
  {
    ProfScope prof("shuffle_count_kernel", s);
    shuffle_count_kernel<<<blocks, kWarps * 32, smem_count, s>>>(p, counts->as<int32_t>());
    after_launch("shuffle_count_kernel");
    prof.stop(static_cast<double>(n) * 4.0 * p.n_keys + static_cast<double>(cells) * 4.0);
  }
  exclusive_scan_i32(counts->as<int32_t>(), starts->as<int32_t>(), cells, s);

  // Output columns: fixed-width ones scattered by the kernel (in groups of
  // kShufMaxFixed, the ranking repeated per group), utf8 ones gathered
  // through the inverse permutation.
  std::vector<ColumnPtr> out(in->num_columns());
  std::vector<int> fixed, utf8;
  for (int i = 0; i < in->num_columns(); ++i) (in->column(i)->type == DType::Utf8 ? utf8 : fixed).push_back(i);
  BufferPtr inverse;
  if (!utf8.empty()) inverse = make_buffer(n * 4, s);
  size_t at = 0;
  do {
    ShufScatter q;
    std::memset(&q, 0, sizeof(q));
    q.starts = starts->as<int32_t>();
    const size_t take = std::min<size_t>(kShufMaxFixed, fixed.size() - at);
    for (size_t j = 0; j < take; ++j) {
      const auto& c = in->column(fixed[at + j]);
      const int w = dtype_width(c->type);
      auto buf = make_buffer(n * w, s);
      q.src[j] = c->data;
      q.dst[j] = buf->data();
      q.width[j] = static_cast<int8_t>(w);
      out[fixed[at + j]] = make_fixed_column(c->type, n, buf);
    }
    q.n_fixed = static_cast<int32_t>(take);
    if (at == 0 && inverse) q.inverse = inverse->as<int32_t>();
    ProfScope prof("shuffle_scatter_kernel", s);
    shuffle_scatter_kernel<<<blocks, kWarps * 32, smem_scatter, s>>>(p, q);
    after_launch("shuffle_scatter_kernel");
    double bytes = static_cast<double>(n) * 4.0 * p.n_keys + (q.inverse ? n * 4.0 : 0.0);
    for (size_t j = 0; j < take; ++j) bytes += 2.0 * n * q.width[j];
    prof.stop(bytes);
    at += take;
  } while (at < fixed.size());
  if (!utf8.empty()) {
    std::vector<GatherSpec> specs;
    for (int i : utf8) specs.push_back(GatherSpec{in->column(i).get(), inverse->as<int32_t>()});
    auto g = gather_columns(specs, n, s);
    for (size_t j = 0; j < utf8.size(); ++j) out[utf8[j]] = g[j];
  }

  // Slot boundaries: the scanned count of each slot's first sub-range.
  std::vector<int32_t> first(num_slots);
  GF_CUDA(cudaMemcpy2DAsync(first.data(), 4, starts->as<int32_t>(), static_cast<size_t>(p.ntiles) * 4, 4,
                            static_cast<size_t>(num_slots), cudaMemcpyDeviceToHost, s));
  sync(s);
  for (int64_t i = 0; i < num_slots; ++i) r.offsets[i] = first[i];
  r.rows = TupleSet::make(in->fields(), std::move(out), n);
  return r;
}

TupleSetPtr slice_rows(const TupleSetPtr& ts, int64_t at, int64_t len) {
  std::vector<ColumnPtr> cols;
  for (int i = 0; i < ts->num_columns(); ++i) {
    const auto& c = ts->column(i);
    auto sl = std::make_shared<Column>(*c);
    sl->length = len;
    if (c->valid != nullptr) {
      if (at % 32 != 0) fail(GFPDB_EUNSUPPORTED, "a slice of a nullable column must start at a multiple of 32 rows");
      sl->valid = c->valid + at / 32;
    }
    if (c->type == DType::Utf8) sl->offsets = c->offsets + at;
    else sl->data = static_cast<const char*>(c->data) + at * dtype_width(c->type);
    cols.push_back(sl);
  }
  return TupleSet::make(ts->fields(), std::move(cols), len);
}

}  // namespace gfpdb
