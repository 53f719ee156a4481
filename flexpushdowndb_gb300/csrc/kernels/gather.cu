// Row gathers (fixed-width and utf8), utf8 concatenation and a single-pass
// exclusive prefix sum. These materialise the outputs of join probes, group
// finalisation and utf8 projections, the GPU form of the
// arrow::compute::Take / ArrayAppender work the reference does per row
// (fpdb-executor/src/physical/join/hashjoin/RecordBatchHashJoiner.cpp:83-119).
#include "common.cuh"
#include "launch.h"

#include <algorithm>
#include <cstring>

namespace gfpdb {

namespace {

constexpr int kGatherMax = kMaxCols * 2;

struct GatherFixedParams {
  int64_t n;              // exact count, or the capacity when n_dev is set
  const int64_t* n_dev;   // device count (deferred sizes)
  int32_t n_cols;
  int32_t pad;
  const void* src[kGatherMax];
  void* dst[kGatherMax];
  const int32_t* idx[kGatherMax];
  int32_t width[kGatherMax];
};

__global__ void __launch_bounds__(256) gather_fixed_kernel(const __grid_constant__ GatherFixedParams p) {
  const int64_t n = clamp_rows(p.n_dev, p.n);
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
    for (int c = 0; c < p.n_cols; ++c) {
      const int32_t i = __ldg(p.idx[c] + r);  // -1: a null (outer joins), stored as 0
      // streaming (evict-first) stores: the gathered rows should not push
      // the gathered-from columns out of the L2
      if (p.width[c] == 8) {
        __stcs(static_cast<long long*>(p.dst[c]) + r, i < 0 ? 0ll : __ldg(static_cast<const long long*>(p.src[c]) + i));
      } else {
        __stcs(static_cast<int*>(p.dst[c]) + r, i < 0 ? 0 : __ldg(static_cast<const int*>(p.src[c]) + i));
      }
    }
  }
}

__global__ void utf8_lengths_kernel(const int32_t* __restrict__ offs, const int32_t* __restrict__ idx,
                                    int32_t* __restrict__ len, int64_t n) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
    const int32_t i = idx[r];
    len[r] = i < 0 ? 0 : offs[i + 1] - offs[i];
  }
}

__global__ void validity_from_index_kernel(const int32_t* __restrict__ idx, int64_t n, uint32_t* __restrict__ out) {
  const int64_t words = (n + 31) / 32;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t w = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; w < words; w += stride) {
    uint32_t bits = 0;
    for (int k = 0; k < 32 && w * 32 + k < n; ++k) bits |= static_cast<uint32_t>(idx[w * 32 + k] >= 0) << k;
    out[w] = bits;
  }
}

// Rows [0, n) of `src` (null: all valid) to rows [at, at + n) of `out`
// (zeroed beforehand; words shared with a neighbouring part take atomicOr).
__global__ void validity_copy_kernel(const uint32_t* __restrict__ src, int64_t n, int64_t at, uint32_t* out) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
    const bool v = src == nullptr || ((src[r >> 5] >> (r & 31)) & 1u);
    if (v) atomicOr(out + ((at + r) >> 5), 1u << ((at + r) & 31));
  }
}

__global__ void utf8_copy_kernel(const int32_t* __restrict__ src_offs, const uint8_t* __restrict__ src_bytes,
                                 const int32_t* __restrict__ idx, const int32_t* __restrict__ dst_offs,
                                 uint8_t* __restrict__ dst_bytes, int64_t n) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
    const int32_t i = idx[r];
    if (i < 0) continue;
    const int32_t b = src_offs[i];
    const int32_t len = src_offs[i + 1] - b;
    const int32_t o = dst_offs[r];
    for (int32_t k = 0; k < len; ++k) dst_bytes[o + k] = src_bytes[b + k];
  }
}

__global__ void rebase_offsets_kernel(const int32_t* __restrict__ src, int32_t* __restrict__ dst, int64_t n,
                                      int32_t sub, int32_t add) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride)
    dst[r] = src[r] - sub + add;
}

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads)
    scan_i32_kernel(const int32_t* __restrict__ in, int32_t* __restrict__ out, int64_t n, int64_t n_tiles,
                    uint64_t* tile_status, uint32_t* ticket, DevStatus* st) {
  __shared__ int s_warp[kScanThreads / 32 + 1];
  __shared__ uint32_t s_tile;
  __shared__ uint64_t s_base;
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const int64_t tile = s_tile;
    if (tile >= n_tiles) break;
    const int64_t row0 = tile * kScanTile + static_cast<int64_t>(threadIdx.x) * kScanItems;
    int v[kScanItems];
    int sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      v[k] = row0 + k < n ? in[row0 + k] : 0;
      sum += v[k];
    }
    int total;
    int excl = block_exclusive_sum<kScanThreads>(sum, &total, s_warp);
    if (threadIdx.x < 32) {
      uint64_t b = lookback_exclusive(tile_status, tile, static_cast<uint64_t>(total), st);
      if (threadIdx.x == 0) s_base = b;
    }
    __syncthreads();
    int64_t run = static_cast<int64_t>(s_base) + excl;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      if (row0 + k < n) out[row0 + k] = static_cast<int32_t>(run);
      run += v[k];
    }
    if (tile == n_tiles - 1 && threadIdx.x == 0) {
      st->value = static_cast<int64_t>(s_base) + total;
      out[n] = static_cast<int32_t>(s_base + total);
    }
    __syncthreads();
  }
}

constexpr int kPackMax = 128;

struct PackParams {
  int32_t n;
  int32_t pad;
  char* dst;
  CopySpan spans[kPackMax];
};

__global__ void __launch_bounds__(256) pack_spans_kernel(const __grid_constant__ PackParams p) {
  const CopySpan& sp = p.spans[blockIdx.x];
  const char* __restrict__ src = static_cast<const char*>(sp.src);
  char* __restrict__ dst = p.dst + sp.dst_off;
  // 16-byte words while both ends are aligned (spans start 256-byte aligned
  // on both sides in practice), four loads in flight per thread, then the
  // tail under 16 bytes
  const bool vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0;
  const int64_t n16 = vec ? sp.bytes / 16 : 0;
  const uint4* s4 = reinterpret_cast<const uint4*>(src);
  uint4* d4 = reinterpret_cast<uint4*>(dst);
  int64_t i = threadIdx.x;
  for (; i + 3 * 256 < n16; i += 4 * 256) {
    const uint4 a = s4[i], b = s4[i + 256], c = s4[i + 512], d = s4[i + 768];
    d4[i] = a;
    d4[i + 256] = b;
    d4[i + 512] = c;
    d4[i + 768] = d;
  }
  for (; i < n16; i += 256) d4[i] = s4[i];
  for (int64_t j = n16 * 16 + threadIdx.x; j < sp.bytes; j += 256) dst[j] = src[j];
}

// Host-to-device copy done by the SMs: each thread streams 16-byte words from
// page-locked host memory (reachable from the device through its unified
// address) into device memory, four loads in flight per thread.
__global__ void __launch_bounds__(256) h2d_copy_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst,
                                                       int64_t n16) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n16; i += 4 * stride) {
    const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
    dst[i] = a;
    dst[i + stride] = b;
    dst[i + 2 * stride] = c;
    dst[i + 3 * stride] = d;
  }
  for (; i < n16; i += stride) dst[i] = src[i];
}

int grid_for(int64_t n, int threads) {
  int64_t blocks = (n + threads - 1) / threads;
  int64_t cap = static_cast<int64_t>(num_sms()) * 8;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return static_cast<int>(blocks);
}

}  // namespace

void copy_h2d(void* dst, const void* src, int64_t bytes, cudaStream_t s) {
  if (bytes <= 0) return;
  const bool aligned = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0;
  cudaPointerAttributes attr{};
  const bool pinned = cudaPointerGetAttributes(&attr, src) == cudaSuccess && attr.type == cudaMemoryTypeHost;
  (void)cudaGetLastError();
  if (host_copy_mode() != 1 || !aligned || !pinned || bytes < (int64_t{1} << 20)) {
    memcpy_h2d(dst, src, bytes, s);
    return;
  }
  const int64_t n16 = bytes / 16;
  const int grid = num_sms() * 4;
  h2d_copy_kernel<<<grid, 256, 0, s>>>(static_cast<const uint4*>(attr.devicePointer ? attr.devicePointer : src),
                                       static_cast<uint4*>(dst), n16);
  after_launch("h2d_copy_kernel");
  const int64_t tail = bytes - n16 * 16;
  if (tail > 0) GF_CUDA(cudaMemcpyAsync(static_cast<char*>(dst) + n16 * 16, static_cast<const char*>(src) + n16 * 16,
                                        tail, cudaMemcpyHostToDevice, s));
  copy_counters().h2d += bytes;
}

void pack_spans(const std::vector<CopySpan>& spans, void* dst, cudaStream_t s) {
  for (size_t at = 0; at < spans.size(); at += kPackMax) {
    PackParams p;
    std::memset(&p, 0, sizeof(p));
    p.dst = static_cast<char*>(dst);
    p.n = static_cast<int32_t>(std::min(spans.size() - at, static_cast<size_t>(kPackMax)));
    for (int i = 0; i < p.n; ++i) p.spans[i] = spans[at + i];
    pack_spans_kernel<<<p.n, 256, 0, s>>>(p);  // 256 threads: the kernel's strides assume it
    after_launch("pack_spans_kernel");
  }
}

namespace {

struct FillParams {
  uint4* dst[2];
  int64_t n16[2];
  uint32_t word[2];
  int32_t n;
};

__global__ void __launch_bounds__(256) fill_regions_kernel(const __grid_constant__ FillParams p) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int r = 0; r < p.n; ++r) {
    const uint4 v = make_uint4(p.word[r], p.word[r], p.word[r], p.word[r]);
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < p.n16[r]; i += stride)
      p.dst[r][i] = v;
  }
}

}  // namespace

void fill_regions(const FillSpan* spans, int n, cudaStream_t s, int max_blocks) {
  FillParams p{};
  int64_t total = 0;
  for (int i = 0; i < n; ++i) {
    if (spans[i].bytes <= 0) continue;
    if (((reinterpret_cast<uintptr_t>(spans[i].dst) | static_cast<uintptr_t>(spans[i].bytes)) & 15u) != 0)
      fail(GFPDB_EINVAL, "fill_regions wants 16-byte aligned regions");
    if (p.n == 2) fail(GFPDB_EINVAL, "fill_regions fills two regions at most");
    p.dst[p.n] = static_cast<uint4*>(spans[i].dst);
    p.n16[p.n] = spans[i].bytes / 16;
    p.word[p.n] = (spans[i].value & 0xFF) * 0x01010101u;
    total += p.n16[p.n];
    ++p.n;
  }
  if (p.n == 0) return;
  int64_t blocks = (total + 255) / 256;
  const int64_t cap = max_blocks > 0 ? max_blocks : static_cast<int64_t>(num_sms()) * 4;
  if (blocks > cap) blocks = cap;
  fill_regions_kernel<<<static_cast<int>(blocks < 1 ? 1 : blocks), 256, 0, s>>>(p);
  after_launch("fill_regions_kernel");
}

void exclusive_scan_i32_async(const int32_t* in, int32_t* out, int64_t n, DevStatus* st, cudaStream_t s) {
  if (n == 0) {
    GF_CUDA(cudaMemsetAsync(out, 0, 4, s));
    return;
  }
  const int64_t n_tiles = (n + kScanTile - 1) / kScanTile;
  auto scratch = make_filled(64 + n_tiles * 8, 0, s);  // ticket line, then the tile words
  uint32_t* ticket = scratch->as<uint32_t>();
  uint64_t* tiles = reinterpret_cast<uint64_t*>(scratch->as<char>() + 64);
  int grid = static_cast<int>(n_tiles < num_sms() * 4 ? n_tiles : num_sms() * 4);
  scan_i32_kernel<<<grid, kScanThreads, 0, s>>>(in, out, n, n_tiles, tiles, ticket, st);
  after_launch("scan_i32_kernel");
}  // scratch is freed stream-ordered, after the scan

int64_t exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, cudaStream_t s) {
  if (n == 0) {
    GF_CUDA(cudaMemsetAsync(out, 0, 4, s));
    return 0;
  }
  const int64_t n_tiles = (n + kScanTile - 1) / kScanTile;
  // scratch: status block, ticket, tile words
  auto scratch = make_filled(sizeof(DevStatus) + 64 + n_tiles * 8, 0, s);
  char* base = scratch->as<char>();
  DevStatus* st = reinterpret_cast<DevStatus*>(base);
  uint32_t* ticket = reinterpret_cast<uint32_t*>(base + sizeof(DevStatus));
  uint64_t* tiles = reinterpret_cast<uint64_t*>(base + sizeof(DevStatus) + 64);
  int grid = static_cast<int>(n_tiles < num_sms() * 4 ? n_tiles : num_sms() * 4);
  scan_i32_kernel<<<grid, kScanThreads, 0, s>>>(in, out, n, n_tiles, tiles, ticket, st);
  after_launch("scan_i32_kernel");
  DevStatus hs;
  GF_CUDA(cudaMemcpyAsync(&hs, st, sizeof(hs), cudaMemcpyDeviceToHost, s));
  sync(s);
  raise_device_status(hs, "prefix sum");
  if (hs.value > INT32_MAX) fail(GFPDB_EUNSUPPORTED, "utf8 column exceeds 2 GiB of bytes");
  return hs.value;
}

std::vector<ColumnPtr> gather_columns(const std::vector<GatherSpec>& specs, int64_t n, cudaStream_t s,
                                      const int64_t* n_dev, BufferPtr n_owner) {
  std::vector<ColumnPtr> out(specs.size());
  GatherFixedParams p;
  std::memset(&p, 0, sizeof(p));
  p.n = n;
  p.n_dev = n_dev;
  bool has_utf8 = false;
  for (auto& sp : specs) has_utf8 |= sp.src->type == DType::Utf8;
  if (has_utf8 && n_dev != nullptr) {
    // utf8 outputs are sized from the exact count
    int64_t exact = 0;
    GF_CUDA(cudaMemcpyAsync(&exact, n_dev, sizeof(exact), cudaMemcpyDeviceToHost, s));
    sync(s);
    p.n = n = exact < n ? exact : n;
    p.n_dev = n_dev = nullptr;
  }
  std::vector<std::pair<size_t, BufferPtr>> fixed;
  for (size_t i = 0; i < specs.size(); ++i) {
    const Column& c = *specs[i].src;
    if (c.type == DType::Utf8) continue;
    int w = dtype_width(c.type);
    auto buf = make_buffer(n * w, s);
    if (p.n_cols >= kGatherMax) fail(GFPDB_EUNSUPPORTED, "too many columns to gather");
    p.src[p.n_cols] = c.data;
    p.dst[p.n_cols] = buf->data();
    p.idx[p.n_cols] = specs[i].idx;
    p.width[p.n_cols] = w;
    ++p.n_cols;
    out[i] = make_fixed_column(c.type, n, buf);
  }
  if (p.n_cols > 0 && n > 0) {
    ProfScope prof("gather_fixed_kernel", s);
    gather_fixed_kernel<<<grid_for(n, 256), 256, 0, s>>>(p);
    after_launch("gather_fixed_kernel");
    double w = 0;
    for (int c = 0; c < p.n_cols; ++c) w += 2.0 * p.width[c] + 4.0;
    prof.stop(static_cast<double>(n) * w);
    if (n_dev) prof.set_bytes_model(nullptr, 0, 0, n_dev, w, n_owner);
  }
  for (size_t i = 0; i < specs.size(); ++i) {
    const Column& c = *specs[i].src;
    if (c.type != DType::Utf8) continue;
    auto offs = make_buffer((n + 1) * 4, s);
    int64_t total = 0;
    if (n > 0) {
      auto lens = make_buffer(n * 4, s);
      utf8_lengths_kernel<<<grid_for(n, 256), 256, 0, s>>>(c.offsets, specs[i].idx, lens->as<int32_t>(), n);
      after_launch("utf8_lengths_kernel");
      total = exclusive_scan_i32(lens->as<int32_t>(), offs->as<int32_t>(), n, s);
    } else {
      GF_CUDA(cudaMemsetAsync(offs->data(), 0, 4, s));
    }
    auto bytes = make_buffer(total, s);
    if (n > 0 && total > 0) {
      utf8_copy_kernel<<<grid_for(n, 256), 256, 0, s>>>(c.offsets, static_cast<const uint8_t*>(c.data),
                                                       specs[i].idx, offs->as<int32_t>(), bytes->as<uint8_t>(), n);
      after_launch("utf8_copy_kernel");
    }
    out[i] = make_utf8_column(n, offs, bytes);
  }
  for (size_t i = 0; i < specs.size(); ++i)
    if (specs[i].may_be_null) out[i] = with_validity(out[i], validity_from_index(specs[i].idx, n, s));
  return out;
}

BufferPtr validity_from_index(const int32_t* idx, int64_t n, cudaStream_t s) {
  const int64_t words = (n + 31) / 32;
  auto bits = make_buffer((words > 0 ? words : 1) * 4, s);
  if (words > 0) {
    validity_from_index_kernel<<<grid_for(words, 256), 256, 0, s>>>(idx, n, bits->as<uint32_t>());
    after_launch("validity_from_index_kernel");
  }
  return bits;
}

BufferPtr validity_concat(const std::vector<std::pair<const uint32_t*, int64_t>>& parts, int64_t total,
                          cudaStream_t s) {
  const int64_t words = (total + 31) / 32;
  auto bits = make_filled((words > 0 ? words : 1) * 4, 0, s);
  int64_t at = 0;
  for (const auto& p : parts) {
    if (p.second > 0) {
      validity_copy_kernel<<<grid_for(p.second, 256), 256, 0, s>>>(p.first, p.second, at, bits->as<uint32_t>());
      after_launch("validity_copy_kernel");
    }
    at += p.second;
  }
  return bits;
}

ColumnPtr null_column(DType t, int64_t n, cudaStream_t s) {
  auto bits = make_filled(((n + 31) / 32 > 0 ? (n + 31) / 32 : 1) * 4, 0, s);
  if (t == DType::Utf8)
    return with_validity(make_utf8_column(n, make_filled((n + 1) * 4, 0, s), make_buffer(0, s)), bits);
  return with_validity(make_fixed_column(t, n, make_filled(n * dtype_width(t) > 0 ? n * dtype_width(t) : 8, 0, s)),
                       bits);
}

ColumnPtr concat_utf8(const std::vector<const Column*>& parts, cudaStream_t s) {
  int64_t n = 0;
  std::vector<std::pair<int32_t, int32_t>> ends(parts.size());
  for (size_t i = 0; i < parts.size(); ++i) {
    n += parts[i]->length;
    int32_t e[2] = {0, 0};
    if (parts[i]->length > 0) {
      GF_CUDA(cudaMemcpyAsync(&e[0], parts[i]->offsets, 4, cudaMemcpyDeviceToHost, s));
      GF_CUDA(cudaMemcpyAsync(&e[1], parts[i]->offsets + parts[i]->length, 4, cudaMemcpyDeviceToHost, s));
    }
    sync(s);
    ends[i] = {e[0], e[1]};
  }
  int64_t total = 0;
  for (auto& e : ends) total += e.second - e.first;
  if (total > INT32_MAX) fail(GFPDB_EUNSUPPORTED, "utf8 column exceeds 2 GiB of bytes");
  auto offs = make_buffer((n + 1) * 4, s);
  auto bytes = make_buffer(total, s);
  int64_t row = 0;
  int32_t at = 0;
  for (size_t i = 0; i < parts.size(); ++i) {
    const Column* c = parts[i];
    if (c->length > 0) {
      rebase_offsets_kernel<<<grid_for(c->length, 256), 256, 0, s>>>(c->offsets, offs->as<int32_t>() + row,
                                                                     c->length, ends[i].first, at);
      after_launch("rebase_offsets_kernel");
      int32_t nb = ends[i].second - ends[i].first;
      if (nb > 0)
        GF_CUDA(cudaMemcpyAsync(bytes->as<char>() + at, static_cast<const char*>(c->data) + ends[i].first, nb,
                                cudaMemcpyDeviceToDevice, s));
      at += nb;
      row += c->length;
    }
  }
  GF_CUDA(cudaMemcpyAsync(offs->as<int32_t>() + n, &at, 4, cudaMemcpyHostToDevice, s));
  sync(s);  // `at` lives on this stack frame
  return make_utf8_column(n, offs, bytes);
}

}  // namespace gfpdb
