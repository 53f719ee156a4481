// Delimited-text ingest into typed device columns.
//
// Replaces CSVReader::read and the reference's SIMD CSV path
// (fpdb-tuple/src/csv/CSVReader.cpp:15-103; find_indexes at
// fpdb-tuple/src/arrow/SIMDParserHelpers.cpp:13-201; per-field std::stoi /
// std::stol / date parsing and ArrayBuilder appends at
// fpdb-tuple/src/arrow/CSVToArrowSIMDChunkParser.cpp:183-313). Parsing rules:
// fields split on the delimiter, rows on '\n' (a trailing '\r' is dropped),
// an optional header line is skipped, and a field wrapped in double quotes
// has the quotes removed (the reference strips surrounding quotes through
// startEndOffsets_, CSVToArrowSIMDChunkParser.cpp:371-373).
//
// Types: int32 / int64 (optional sign, decimal digits), decimal(p, s) text
// into int64 scaled by 10^s with exact integer arithmetic (the reference reads
// decimals as double; here they are exact cents), date32 from YYYY-MM-DD
// (days since 1970-01-01 by Howard Hinnant's public-domain days_from_civil
// algorithm), and utf8 (bytes copied as they are).
//
// Kernels: (1) newline count per 64 KiB tile, (2) prefix sum, (3) row start
// offsets, written in input order with one block scan per 4 KiB step,
// (4) per block of 256 rows: each thread splits its row into field offsets in
// shared memory, then the block converts fields column by column so output
// stores are coalesced; utf8 fields record their length and start, and
// (5) after a prefix sum of the lengths, a copy kernel moves the bytes.
#include <cstring>

#include "common.cuh"
#include "launch.h"

namespace gfpdb {

namespace {

constexpr int kCsvThreads = 256;
constexpr int kCsvTileBytes = 65536;
constexpr int kStepBytes = kCsvThreads * 16;

__global__ void __launch_bounds__(kCsvThreads)
    csv_newline_count_kernel(const uint8_t* __restrict__ text, int64_t n, int32_t* __restrict__ counts) {
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kCsvTileBytes;
  int c = 0;
  for (int step = 0; step < kCsvTileBytes / kStepBytes; ++step) {
    const int64_t at = base + static_cast<int64_t>(step) * kStepBytes + threadIdx.x * 16;
    if (at + 16 <= n) {
      const uint4 v = __ldg(reinterpret_cast<const uint4*>(text + at));
      const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        // bytes equal to '\n' (0x0A): classic has-zero-byte test on w ^ 0x0A0A0A0A
        const uint32_t x = w[k] ^ 0x0A0A0A0Au;
        const uint32_t z = (x - 0x01010101u) & ~x & 0x80808080u;
        // The test can flag a 0x0B byte right after a real match; count exactly instead.
        if (z != 0) {
#pragma unroll
          for (int b = 0; b < 4; ++b) c += ((w[k] >> (8 * b)) & 0xFFu) == 0x0Au;
        }
      }
    } else {
      for (int64_t i = at; i < at + 16 && i < n; ++i) c += text[i] == '\n';
    }
  }
  __shared__ int s_warp[kCsvThreads / 32 + 1];
  int total;
  (void)block_exclusive_sum<kCsvThreads>(c, &total, s_warp);
  if (threadIdx.x == 0) counts[blockIdx.x] = total;
}

// Writes the byte offset just after each '\n' (the start of the next row).
__global__ void __launch_bounds__(kCsvThreads)
    csv_row_starts_kernel(const uint8_t* __restrict__ text, int64_t n, const int32_t* __restrict__ tile_offsets,
                          int64_t* __restrict__ starts) {
  __shared__ int s_warp[kCsvThreads / 32 + 1];
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kCsvTileBytes;
  int64_t run = tile_offsets[blockIdx.x];
  for (int step = 0; step < kCsvTileBytes / kStepBytes; ++step) {
    const int64_t at = base + static_cast<int64_t>(step) * kStepBytes + threadIdx.x * 16;
    uint32_t mask = 0;
    for (int b = 0; b < 16; ++b)
      if (at + b < n && text[at + b] == '\n') mask |= 1u << b;
    int total;
    const int excl = block_exclusive_sum<kCsvThreads>(__popc(mask), &total, s_warp);
    int64_t o = run + excl;
    while (mask) {
      const int b = __ffs(mask) - 1;
      mask &= mask - 1;
      starts[o++] = at + b + 1;
    }
    run += total;
    __syncthreads();
  }
}

__device__ __forceinline__ int32_t days_from_civil(int32_t y, uint32_t m, uint32_t d) {
  y -= m <= 2;
  const int32_t era = (y >= 0 ? y : y - 399) / 400;
  const uint32_t yoe = static_cast<uint32_t>(y - era * 400);
  const uint32_t doy = (153 * (m + (m > 2 ? -3 : 9)) + 2) / 5 + d - 1;
  const uint32_t doe = yoe * 365 + yoe / 4 - yoe / 100 + doy;
  return era * 146097 + static_cast<int32_t>(doe) - 719468;
}

struct CsvOut {
  void* data;         // fixed-width output, or utf8 lengths (int32)
  int64_t* str_start; // utf8: absolute start offset of each field
  int32_t field;      // field index in the line
  int32_t type;       // ColTypeCode
  int32_t decimal;    // 1: decimal text -> scaled int64
  int32_t scale;
};

constexpr int kCsvMaxOut = 32;

struct CsvParams {
  const uint8_t* text;
  const int64_t* starts;  // n_rows + 1 row starts (last = end of text + 1)
  int64_t n_rows;
  int32_t n_fields;
  int32_t n_out;
  uint8_t delim;
  uint8_t pad[7];
  DevStatus* st;
  CsvOut out[kCsvMaxOut];
};

__device__ __forceinline__ void trim_quotes(const uint8_t* text, int64_t& b, int64_t& e) {
  if (e - b >= 2 && text[b] == '"' && text[e - 1] == '"') {
    ++b;
    --e;
  }
}

__device__ __forceinline__ bool parse_int(const uint8_t* t, int64_t b, int64_t e, int64_t* v) {
  if (b >= e) return false;
  bool neg = false;
  if (t[b] == '-' || t[b] == '+') {
    neg = t[b] == '-';
    ++b;
  }
  if (b >= e) return false;
  uint64_t acc = 0;
  for (int64_t i = b; i < e; ++i) {
    const uint32_t d = static_cast<uint32_t>(t[i]) - '0';
    if (d > 9) return false;
    acc = acc * 10 + d;
  }
  *v = neg ? static_cast<int64_t>(0ull - acc) : static_cast<int64_t>(acc);
  return true;
}

__device__ __forceinline__ bool parse_decimal(const uint8_t* t, int64_t b, int64_t e, int scale, int64_t* v) {
  if (b >= e) return false;
  bool neg = false;
  if (t[b] == '-' || t[b] == '+') {
    neg = t[b] == '-';
    ++b;
  }
  uint64_t acc = 0;
  int frac = -1;  // digits seen after the point, -1 before it
  bool any = false;
  for (int64_t i = b; i < e; ++i) {
    const uint8_t c = t[i];
    if (c == '.') {
      if (frac >= 0) return false;
      frac = 0;
      continue;
    }
    const uint32_t d = static_cast<uint32_t>(c) - '0';
    if (d > 9) return false;
    if (frac >= 0) {
      if (frac == scale) return false;  // more fractional digits than the scale holds
      ++frac;
    }
    acc = acc * 10 + d;
    any = true;
  }
  if (!any) return false;
  for (int k = frac < 0 ? 0 : frac; k < scale; ++k) acc *= 10;
  *v = neg ? static_cast<int64_t>(0ull - acc) : static_cast<int64_t>(acc);
  return true;
}

__device__ __forceinline__ bool parse_date(const uint8_t* t, int64_t b, int64_t e, int32_t* v) {
  if (e - b != 10 || t[b + 4] != '-' || t[b + 7] != '-') return false;
  int32_t y = 0;
  uint32_t m = 0, d = 0;
  for (int i = 0; i < 4; ++i) {
    const uint32_t x = static_cast<uint32_t>(t[b + i]) - '0';
    if (x > 9) return false;
    y = y * 10 + static_cast<int32_t>(x);
  }
  for (int i = 5; i < 7; ++i) {
    const uint32_t x = static_cast<uint32_t>(t[b + i]) - '0';
    if (x > 9) return false;
    m = m * 10 + x;
  }
  for (int i = 8; i < 10; ++i) {
    const uint32_t x = static_cast<uint32_t>(t[b + i]) - '0';
    if (x > 9) return false;
    d = d * 10 + x;
  }
  if (m < 1 || m > 12 || d < 1 || d > 31) return false;
  *v = days_from_civil(y, m, d);
  return true;
}

__global__ void __launch_bounds__(kCsvThreads) csv_convert_kernel(const __grid_constant__ CsvParams p) {
  extern __shared__ int32_t s_fs[];  // [kCsvThreads][n_fields + 1] field starts relative to the row start
  const int F = p.n_fields;
  const int64_t row0 = static_cast<int64_t>(blockIdx.x) * kCsvThreads;
  const int lr = threadIdx.x;
  const int64_t row = row0 + lr;
  // Phase A: split my row.
  if (row < p.n_rows) {
    const int64_t b = p.starts[row];
    int64_t e = p.starts[row + 1] - 1;  // exclusive of the '\n'
    if (e > b && p.text[e - 1] == '\r') --e;
    int32_t* fs = s_fs + lr * (F + 1);
    fs[0] = 0;
    int k = 1;
    for (int64_t i = b; i < e; ++i) {
      if (p.text[i] == p.delim) {
        if (k < F) fs[k] = static_cast<int32_t>(i + 1 - b);
        ++k;
      }
    }
    fs[F] = static_cast<int32_t>(e + 1 - b);
    // A short row leaves its missing fields empty (start = end of row), so
    // phase B never reads outside the row; the row is reported as malformed.
    for (int j = k; j < F; ++j) fs[j] = fs[F];
    if (k != F) raise_status(p.st, GFPDB_EINVAL, static_cast<int32_t>(row < INT32_MAX ? row : INT32_MAX));
  }
  __syncthreads();
  // Phase B: convert, one emitted column at a time across the block's rows.
  const int64_t rows_here = p.n_rows - row0 < kCsvThreads ? p.n_rows - row0 : kCsvThreads;
  for (int task = threadIdx.x; task < p.n_out * kCsvThreads; task += kCsvThreads) {
    const int oc = task / kCsvThreads;
    const int r = task % kCsvThreads;
    if (r >= rows_here) continue;
    const CsvOut& o = p.out[oc];
    const int32_t* fs = s_fs + r * (F + 1);
    const int64_t rb = p.starts[row0 + r];
    int64_t b = rb + fs[o.field];
    int64_t e = rb + fs[o.field + 1] - 1;
    if (e < b) e = b;
    trim_quotes(p.text, b, e);
    const int64_t orow = row0 + r;
    bool ok = true;
    if (o.type == CT_UTF8) {
      static_cast<int32_t*>(o.data)[orow] = static_cast<int32_t>(e - b);
      o.str_start[orow] = b;
    } else if (o.type == CT_DATE32) {
      int32_t v = 0;
      ok = parse_date(p.text, b, e, &v);
      static_cast<int32_t*>(o.data)[orow] = v;
    } else {
      int64_t v = 0;
      ok = o.decimal ? parse_decimal(p.text, b, e, o.scale, &v) : parse_int(p.text, b, e, &v);
      if (o.type == CT_I32) {
        if (v < INT32_MIN || v > INT32_MAX) ok = false;
        static_cast<int32_t*>(o.data)[orow] = static_cast<int32_t>(v);
      } else {
        static_cast<int64_t*>(o.data)[orow] = v;
      }
    }
    if (!ok) raise_status(p.st, GFPDB_EINVAL, static_cast<int32_t>(orow < INT32_MAX ? orow : INT32_MAX));
  }
}

__global__ void csv_copy_strings_kernel(const uint8_t* __restrict__ text, const int64_t* __restrict__ str_start,
                                        const int32_t* __restrict__ offs, uint8_t* __restrict__ out, int64_t n) {
  // one warp per row: lanes copy consecutive bytes
  const int lane = threadIdx.x & 31;
  const int64_t w = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t r = w; r < n; r += nw) {
    const int64_t s = str_start[r];
    const int32_t o = offs[r], len = offs[r + 1] - o;
    for (int32_t k = lane; k < len; k += 32) out[o + k] = text[s + k];
  }
}

__global__ void csv_tail_kernel(int64_t* starts, int64_t at, int64_t value) { starts[at] = value; }

}  // namespace

TupleSetPtr csv_parse(const char* device_text, int64_t n_bytes, char delimiter, bool has_header,
                      const std::vector<CsvField>& fields, const std::vector<int>& emit, cudaStream_t s) {
  if (fields.empty()) fail(GFPDB_EINVAL, "CSV schema has no fields");
  if (static_cast<int>(emit.size()) > kCsvMaxOut) fail(GFPDB_EUNSUPPORTED, "too many CSV columns to emit");
  if (static_cast<int>(fields.size()) > 256) fail(GFPDB_EUNSUPPORTED, "too many CSV fields per line");
  if (n_bytes >= (int64_t{1} << 40)) fail(GFPDB_EUNSUPPORTED, "CSV text too large");
  const uint8_t* text = reinterpret_cast<const uint8_t*>(device_text);
  if ((reinterpret_cast<uintptr_t>(text) & 15u) != 0) fail(GFPDB_EINVAL, "CSV text must be 16-byte aligned");

  // (1)-(3): row starts
  const int64_t n_tiles = n_bytes > 0 ? (n_bytes + kCsvTileBytes - 1) / kCsvTileBytes : 0;
  auto counts = make_buffer((n_tiles + 1) * 4, s);
  auto tile_off = make_buffer((n_tiles + 1) * 4, s);
  int64_t newlines = 0;
  if (n_tiles > 0) {
    ProfScope prof("csv_newline_count_kernel", s);
    csv_newline_count_kernel<<<static_cast<int>(n_tiles), kCsvThreads, 0, s>>>(text, n_bytes, counts->as<int32_t>());
    after_launch("csv_newline_count_kernel");
    prof.stop(static_cast<double>(n_bytes));
    newlines = exclusive_scan_i32(counts->as<int32_t>(), tile_off->as<int32_t>(), n_tiles, s);
  }
  // Last line without a trailing newline still counts as a row.
  char last = '\n';
  if (n_bytes > 0) {
    GF_CUDA(cudaMemcpyAsync(&last, device_text + n_bytes - 1, 1, cudaMemcpyDeviceToHost, s));
    sync(s);
  }
  const int64_t lines = newlines + (last != '\n' ? 1 : 0);
  // starts[0] = 0, starts[1 + k] = after the k-th newline; an extra entry
  // closes an unterminated last line.
  auto starts = make_buffer((lines + 2) * 8, s);
  GF_CUDA(cudaMemsetAsync(starts->data(), 0, 8, s));
  if (n_tiles > 0) {
    ProfScope prof("csv_row_starts_kernel", s);
    csv_row_starts_kernel<<<static_cast<int>(n_tiles), kCsvThreads, 0, s>>>(text, n_bytes, tile_off->as<int32_t>(),
                                                                           starts->as<int64_t>() + 1);
    after_launch("csv_row_starts_kernel");
    prof.stop(static_cast<double>(n_bytes) + 8.0 * static_cast<double>(newlines));
  }
  if (last != '\n') {
    csv_tail_kernel<<<1, 1, 0, s>>>(starts->as<int64_t>(), lines, n_bytes + 1);
    after_launch("csv_tail_kernel");
  }
  const int64_t skip = has_header && lines > 0 ? 1 : 0;
  const int64_t n_rows = lines - skip;
  const int64_t* row_starts = starts->as<int64_t>() + skip;

  // (4) convert
  std::vector<Field> out_fields;
  std::vector<BufferPtr> bufs(emit.size()), sstart(emit.size());
  CsvParams* pp = new CsvParams;
  std::unique_ptr<CsvParams> holder(pp);
  CsvParams& p = *pp;
  std::memset(&p, 0, sizeof(p));
  p.text = text;
  p.starts = row_starts;
  p.n_rows = n_rows;
  p.n_fields = static_cast<int32_t>(fields.size());
  p.n_out = static_cast<int32_t>(emit.size());
  p.delim = static_cast<uint8_t>(delimiter);
  auto status = make_buffer(sizeof(DevStatus), s);
  GF_CUDA(cudaMemsetAsync(status->data(), 0, sizeof(DevStatus), s));
  p.st = status->as<DevStatus>();
  for (size_t k = 0; k < emit.size(); ++k) {
    const CsvField& f = fields[emit[k]];
    out_fields.push_back(Field{f.name, f.type});
    CsvOut& o = p.out[k];
    o.field = emit[k];
    o.type = static_cast<int32_t>(f.type);
    o.decimal = f.decimal ? 1 : 0;
    o.scale = f.scale;
    if (f.type == DType::Utf8) {
      bufs[k] = make_buffer(n_rows * 4, s);  // lengths, then offsets live elsewhere
      sstart[k] = make_buffer(n_rows * 8, s);
      o.str_start = sstart[k]->as<int64_t>();
    } else {
      bufs[k] = make_buffer(n_rows * dtype_width(f.type), s);
    }
    o.data = bufs[k]->data();
  }
  if (n_rows > 0) {
    const size_t dyn = static_cast<size_t>(kCsvThreads) * (fields.size() + 1) * 4;
    if (dyn > 48 * 1024) GF_CUDA(cudaFuncSetAttribute(csv_convert_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(dyn)));
    const int64_t blocks = (n_rows + kCsvThreads - 1) / kCsvThreads;
    if (blocks > INT32_MAX) fail(GFPDB_EUNSUPPORTED, "too many CSV rows");
    ProfScope prof("csv_convert_kernel", s);
    csv_convert_kernel<<<static_cast<int>(blocks), kCsvThreads, dyn, s>>>(p);
    after_launch("csv_convert_kernel");
    double out_w = 0;
    for (auto& f : out_fields) out_w += f.type == DType::Utf8 ? 12 : dtype_width(f.type);
    prof.stop(static_cast<double>(n_bytes) + static_cast<double>(n_rows) * out_w);
  }
  DevStatus hs;
  GF_CUDA(cudaMemcpyAsync(&hs, status->data(), sizeof(hs), cudaMemcpyDeviceToHost, s));
  sync(s);
  if (hs.code == GFPDB_EINVAL)
    fail(GFPDB_EINVAL, "malformed CSV field or wrong field count near data row " + std::to_string(hs.detail));
  raise_device_status(hs, "CSV parse");

  // (5) utf8 bytes
  std::vector<ColumnPtr> cols;
  for (size_t k = 0; k < emit.size(); ++k) {
    if (out_fields[k].type != DType::Utf8) {
      cols.push_back(make_fixed_column(out_fields[k].type, n_rows, bufs[k]));
      continue;
    }
    auto offs = make_buffer((n_rows + 1) * 4, s);
    const int64_t total = exclusive_scan_i32(bufs[k]->as<int32_t>(), offs->as<int32_t>(), n_rows, s);
    auto bytes = make_buffer(total, s);
    if (n_rows > 0 && total > 0) {
      int64_t blocks = (n_rows * 32 + 255) / 256;
      int64_t cap = static_cast<int64_t>(num_sms()) * 16;
      ProfScope prof("csv_copy_strings_kernel", s);
      csv_copy_strings_kernel<<<static_cast<int>(blocks < cap ? blocks : cap), 256, 0, s>>>(
          text, sstart[k]->as<int64_t>(), offs->as<int32_t>(), bytes->as<uint8_t>(), n_rows);
      after_launch("csv_copy_strings_kernel");
      prof.stop(2.0 * static_cast<double>(total) + 12.0 * static_cast<double>(n_rows));
    }
    cols.push_back(make_utf8_column(n_rows, offs, bytes));
  }
  return TupleSet::make(std::move(out_fields), std::move(cols), n_rows);
}

}  // namespace gfpdb
