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
// Kernels: the text is cut into 16 KiB tiles of 256 threads x 64 bytes (read
// with 128-bit loads). A separator is a delimiter or a newline; in a
// well-formed text every row has n_fields separators, so the field that ends
// at the g-th separator of the text is row g / n_fields, field g % n_fields.
// (1) csv_index_kernel: per tile, the separator count and the position of its
// last separator; (2) csv_tile_scan_kernel: each tile's first separator
// ordinal and the position of the separator before it; (3) csv_fields_kernel:
// every thread finds the separators of its 64 bytes, ranks them with block
// scans, and converts the field ending at each one (a newline at any
// position but the last field of a row marks the row malformed); utf8 fields
// record their length and start, and (4) after a prefix sum of the lengths a
// copy kernel moves the bytes.
#include <cstring>

#include "common.cuh"
#include "launch.h"

namespace gfpdb {

namespace {

constexpr int kCsvThreads = 256;
constexpr int kCsvChunk = 64;                               // bytes per thread
constexpr int kCsvTile = kCsvThreads * kCsvChunk;           // bytes per tile
constexpr int kCsvScanThreads = 1024;

// Block-wide exclusive scan of one int64 per thread under `op` (sum or max)
// with identity `id`; *total gets the reduction over the block.
template <int NT, typename Op>
__device__ __forceinline__ int64_t block_scan64(int64_t x, int64_t id, Op op, int64_t* total, int64_t* s_w) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int NW = NT / 32;
  int64_t incl = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl = op(incl, y);
  }
  if (lane == 31) s_w[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const int64_t w = lane < NW ? s_w[lane] : id;
    int64_t wi = w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, wi, d);
      if (lane >= d) wi = op(wi, y);
    }
    const int64_t prev_w = __shfl_up_sync(0xffffffffu, wi, 1);  // every lane takes part
    if (lane < NW) s_w[NW + 1 + lane] = lane == 0 ? id : prev_w;
    if (lane == NW - 1) s_w[NW] = wi;
  }
  __syncthreads();
  const int64_t up = __shfl_up_sync(0xffffffffu, incl, 1);  // every lane takes part
  const int64_t excl_in_warp = lane == 0 ? id : up;
  const int64_t r = op(s_w[NW + 1 + warp], excl_in_warp);
  *total = s_w[NW];
  __syncthreads();  // s_w is reused by the next scan
  return r;
}

struct SumOp {
  __device__ int64_t operator()(int64_t a, int64_t b) const { return a + b; }
};
struct MaxOp {
  __device__ int64_t operator()(int64_t a, int64_t b) const { return a > b ? a : b; }
};

// The 64 bytes of this thread's chunk (zeros past the end of the text).
__device__ __forceinline__ void load_chunk(const uint8_t* text, int64_t n, int64_t at, uint32_t w[16]) {
  if (at + kCsvChunk <= n) {
    const uint4* q = reinterpret_cast<const uint4*>(text + at);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint4 v = __ldg(q + k);
      w[4 * k] = v.x;
      w[4 * k + 1] = v.y;
      w[4 * k + 2] = v.z;
      w[4 * k + 3] = v.w;
    }
  } else {  // the last chunk: byte loads, indexes fixed at compile time so w stays in registers
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      uint32_t v = 0;
#pragma unroll
      for (int b = 0; b < 4; ++b)
        if (at + 4 * k + b < n) v |= static_cast<uint32_t>(text[at + 4 * k + b]) << (8 * b);
      w[k] = v;
    }
  }
}

// 0x80 in every byte of x that is zero, 0 elsewhere (exact: no carry
// crosses a byte, since (b & 0x7F) + 0x7F <= 0xFE).
__device__ __forceinline__ uint32_t zero_byte_bits(uint32_t x) {
  return ~(((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x | 0x7F7F7F7Fu);
}

// Bits 7, 15, 23, 31 of z to bits 0..3 (the four products land on distinct
// bit positions, so nothing carries into bits 21..24).
__device__ __forceinline__ uint32_t high_bits_to_nibble(uint32_t z) {
  return (((z >> 7) * 0x00204081u) >> 21) & 0xFu;
}

// Bit i set when byte i of the chunk is a separator (delimiter or newline),
// four bytes at a time.
__device__ __forceinline__ uint64_t separator_bits(const uint32_t w[16], uint8_t delim) {
  const uint32_t dpat = static_cast<uint32_t>(delim) * 0x01010101u;
  uint64_t m = 0;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const uint32_t z = zero_byte_bits(w[k] ^ dpat) | zero_byte_bits(w[k] ^ 0x0A0A0A0Au);
    m |= static_cast<uint64_t>(high_bits_to_nibble(z)) << (4 * k);
  }
  return m;
}

// (1) per tile: separators, and the position of the last one (-1: none)
__global__ void __launch_bounds__(kCsvThreads)
    csv_index_kernel(const uint8_t* __restrict__ text, int64_t n, uint8_t delim, int64_t* __restrict__ tile_count,
                     int64_t* __restrict__ tile_last, uint64_t* __restrict__ chunk_masks) {
  __shared__ int64_t s_w[2 * (kCsvThreads / 32) + 2];
  const int64_t at = static_cast<int64_t>(blockIdx.x) * kCsvTile + static_cast<int64_t>(threadIdx.x) * kCsvChunk;
  uint32_t w[16];
  load_chunk(text, n, at, w);
  uint64_t m = separator_bits(w, delim);
  if (at + kCsvChunk > n) m &= n > at ? (~uint64_t{0} >> (64 - (n - at))) : 0;  // bytes past the end
  chunk_masks[at / kCsvChunk] = m;  // one entry per chunk of every tile: kept for csv_fields_kernel
  const int64_t cnt = __popcll(m);
  const int64_t last = m ? at + 63 - __clzll(static_cast<long long>(m)) : -1;
  int64_t total_cnt, max_last;
  (void)block_scan64<kCsvThreads>(cnt, 0, SumOp{}, &total_cnt, s_w);
  (void)block_scan64<kCsvThreads>(last, -1, MaxOp{}, &max_last, s_w);
  if (threadIdx.x == 0) {
    tile_count[blockIdx.x] = total_cnt;
    tile_last[blockIdx.x] = max_last;
  }
}

// (2) one CTA: exclusive sum of the tile counts (in place), exclusive max of
// the tiles' last separators (in place), the total into out[0] and the last
// byte of the text into out[1].
__global__ void __launch_bounds__(kCsvScanThreads)
    csv_tile_scan_kernel(int64_t* __restrict__ tile_count, int64_t* __restrict__ tile_last, int64_t n_tiles,
                         const uint8_t* __restrict__ text, int64_t n, int64_t* __restrict__ out) {
  __shared__ int64_t s_w[2 * (kCsvScanThreads / 32) + 2];
  int64_t carry_sum = 0, carry_max = -1;
  for (int64_t base = 0; base < n_tiles; base += kCsvScanThreads) {
    const int64_t t = base + threadIdx.x;
    const int64_t c = t < n_tiles ? tile_count[t] : 0;
    const int64_t l = t < n_tiles ? tile_last[t] : -1;
    int64_t tot_c, tot_l;
    const int64_t ec = block_scan64<kCsvScanThreads>(c, 0, SumOp{}, &tot_c, s_w);
    const int64_t el = block_scan64<kCsvScanThreads>(l, -1, MaxOp{}, &tot_l, s_w);
    if (t < n_tiles) {
      tile_count[t] = carry_sum + ec;
      tile_last[t] = carry_max > el ? carry_max : el;
    }
    carry_sum += tot_c;
    carry_max = carry_max > tot_l ? carry_max : tot_l;
  }
  if (threadIdx.x == 0) {
    out[0] = carry_sum;
    out[1] = n > 0 ? text[n - 1] : '\n';
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
  int32_t type;       // ColTypeCode
  int32_t decimal;    // 1: decimal text -> scaled int64
  int32_t scale;
  int32_t pad;
};

constexpr int kCsvMaxOut = 32;
constexpr int kCsvMaxFields = 256;

struct CsvParams {
  const uint8_t* text;
  int64_t n;                   // text bytes
  const int64_t* tile_base;    // first separator ordinal of each tile
  const int64_t* tile_prev;    // position of the separator before each tile (-1: none)
  const uint64_t* chunk_masks; // separator bits of every 64-byte chunk (csv_index_kernel)
  int64_t n_rows;              // data rows (after the header)
  int32_t n_fields;
  int32_t header;              // 1: the first row is skipped
  int32_t virtual_end;         // 1: the text does not end with '\n' (a newline is implied at n)
  uint8_t delim;
  uint8_t pad[3];
  DevStatus* st;
  int16_t slot[kCsvMaxFields]; // output slot of each field (-1: not emitted)
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

__device__ __forceinline__ void csv_malformed(DevStatus* st, int64_t row) {
  raise_status(st, GFPDB_EINVAL, static_cast<int32_t>(row < 0 ? 0 : (row < INT32_MAX ? row : INT32_MAX)));
}

// Converts one field, bytes [b, e) of t (t is the text or a shared-memory copy
// of part of it; `shift` turns an index of t into a text offset) into output
// slot sl at `row`.
__device__ __forceinline__ void convert_field(const CsvParams& p, int sl, int64_t row, const uint8_t* t, int64_t b,
                                              int64_t e, int64_t shift, bool is_nl) {
  if (is_nl && e > b && t[e - 1] == '\r') --e;
  trim_quotes(t, b, e);
  const CsvOut& o = p.out[sl];
  bool ok = true;
  if (o.type == CT_UTF8) {
    static_cast<int32_t*>(o.data)[row] = static_cast<int32_t>(e - b);
    o.str_start[row] = b + shift;
  } else if (o.type == CT_DATE32) {
    int32_t v = 0;
    ok = parse_date(t, b, e, &v);
    static_cast<int32_t*>(o.data)[row] = v;
  } else {
    int64_t v = 0;
    ok = o.decimal ? parse_decimal(t, b, e, o.scale, &v) : parse_int(t, b, e, &v);
    if (o.type == CT_I32) {
      if (v < INT32_MIN || v > INT32_MAX) ok = false;
      static_cast<int32_t*>(o.data)[row] = static_cast<int32_t>(v);
    } else {
      static_cast<int64_t*>(o.data)[row] = v;
    }
  }
  if (!ok) csv_malformed(p.st, row);
}

// Separators of one tile kept in shared memory; a tile with more (fields of
// about 4 bytes on average) is converted by the thread-per-chunk loop instead.
constexpr int kCsvSepCap = 4096;
constexpr int kCsvPosSlots = kCsvSepCap + 2 * kCsvMaxFields;

// (3) every field, by the separator that ends it. The tile's text and its
// separator positions go to shared memory, the positions stored by (field,
// row) so that consecutive threads convert one field of consecutive rows: the
// same conversion in every lane and coalesced stores into the column.
__global__ void __launch_bounds__(kCsvThreads) csv_fields_kernel(const __grid_constant__ CsvParams p) {
  __shared__ int64_t s_w[2 * (kCsvThreads / 32) + 2];
  __shared__ __align__(16) uint32_t s_text[kCsvTile / 4];
  __shared__ int32_t s_pos[kCsvPosSlots];  // tile-relative position | (newline ? 1 << 31 : 0)
  const int64_t tile0 = static_cast<int64_t>(blockIdx.x) * kCsvTile;
  const int64_t at = tile0 + static_cast<int64_t>(threadIdx.x) * kCsvChunk;
  uint32_t w[16];
  load_chunk(p.text, p.n, at, w);
  // the separators found by csv_index_kernel (bytes past the end excluded); a
  // separator is a newline when its byte is one
  uint64_t m = p.chunk_masks[at / kCsvChunk];
  // the implied newline after an unterminated last line belongs to the chunk
  // holding the last byte
  const bool has_end = p.virtual_end && p.n > at && p.n <= at + kCsvChunk;
  const int cnt = __popcll(m) + (has_end ? 1 : 0);
  const int64_t last = has_end ? p.n : (m ? at + 63 - __clzll(static_cast<long long>(m)) : -1);
  int64_t tot, unused;
  const int64_t g0 = p.tile_base[blockIdx.x];
  const int64_t first = g0 + block_scan64<kCsvThreads>(cnt, 0, SumOp{}, &tot, s_w);
  const int64_t before = block_scan64<kCsvThreads>(last, -1, MaxOp{}, &unused, s_w);
  const int64_t tile_prev = p.tile_prev[blockIdx.x];
  const int F = p.n_fields;

  if (tot > kCsvSepCap) {  // uniform over the block
    int64_t prev = tile_prev > before ? tile_prev : before;
    int64_t g = first;
    for (int k = 0; k < cnt; ++k, ++g) {
      int64_t pos;
      bool is_nl;
      if (m != 0) {
        const int bit = __ffsll(static_cast<long long>(m)) - 1;
        m &= m - 1;
        pos = at + bit;
        is_nl = p.text[pos] == '\n';
      } else {  // the implied newline
        pos = p.n;
        is_nl = true;
      }
      const int64_t b = prev + 1;
      prev = pos;
      const int col = static_cast<int>(g % F);
      const int64_t row = g / F - p.header;
      if (is_nl != (col == F - 1)) {
        csv_malformed(p.st, row);
        continue;
      }
      if (row < 0 || row >= p.n_rows) continue;
      const int sl = p.slot[col];
      if (sl >= 0) convert_field(p, sl, row, p.text, b, pos, 0, is_nl);
    }
    return;
  }

  {
    uint4* dst = reinterpret_cast<uint4*>(s_text) + threadIdx.x * (kCsvChunk / 16);
#pragma unroll
    for (int k = 0; k < kCsvChunk / 16; ++k) dst[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
  }
  const int64_t row0 = g0 / F;
  const int RS = kCsvSepCap / F + 2;  // rows per field in s_pos; F * RS <= kCsvPosSlots
  if (cnt > 0) {
    const int64_t q = first / F;
    int c = static_cast<int>(first - q * F);
    int r = static_cast<int>(q - row0);
    for (int k = 0; k < cnt; ++k) {
      int32_t rel;
      bool is_nl;
      if (m != 0) {
        const int bit = __ffsll(static_cast<long long>(m)) - 1;
        m &= m - 1;
        rel = static_cast<int32_t>(at - tile0) + bit;
        is_nl = reinterpret_cast<const uint8_t*>(s_text)[rel] == '\n';  // this thread staged that byte
      } else {
        rel = static_cast<int32_t>(p.n - tile0);
        is_nl = true;
      }
      s_pos[c * RS + r] = rel | (is_nl ? INT32_MIN : 0);
      if (++c == F) {
        c = 0;
        ++r;
      }
    }
  }
  __syncthreads();
  if (tot == 0) return;
  const int64_t g_end = g0 + tot;
  const int R = static_cast<int>((g_end - 1) / F - row0 + 1);
  const int items = F * R;
  const uint8_t* st = reinterpret_cast<const uint8_t*>(s_text);
  // item i is field i / R of row i % R; advanced per step of kCsvThreads
  // instead of divided per item
  const int dc = kCsvThreads / R, dr = kCsvThreads - dc * R;
  int c_next = static_cast<int>(threadIdx.x) / R;
  int r_next = static_cast<int>(threadIdx.x) - c_next * R;
  for (int i = threadIdx.x; i < items; i += kCsvThreads) {
    const int c = c_next, r = r_next;
    r_next += dr;
    c_next += dc;
    if (r_next >= R) {
      r_next -= R;
      ++c_next;
    }
    const int64_t g = (row0 + r) * F + c;
    if (g < g0 || g >= g_end) continue;
    const int32_t pe = s_pos[c * RS + r];
    const bool is_nl = pe < 0;
    const int64_t row = row0 + r - p.header;
    if (is_nl != (c == F - 1)) {
      csv_malformed(p.st, row);
      continue;
    }
    if (row < 0 || row >= p.n_rows) continue;
    const int sl = p.slot[c];
    if (sl < 0) continue;
    const int64_t e = pe & INT32_MAX;
    if (g == g0) {  // the field may start before the tile
      const int64_t b = tile_prev + 1;
      if (b >= tile0)
        convert_field(p, sl, row, st, b - tile0, e, tile0, is_nl);
      else
        convert_field(p, sl, row, p.text, b, tile0 + e, 0, is_nl);
    } else {
      const int32_t pb = c > 0 ? s_pos[(c - 1) * RS + r] : s_pos[(F - 1) * RS + r - 1];
      convert_field(p, sl, row, st, (pb & INT32_MAX) + 1, e, tile0, is_nl);
    }
  }
}

// (4) utf8 bytes: each warp takes 32 consecutive rows, whose output bytes are
// one contiguous range, and writes it as whole 32-bit words (four per lane in
// flight), with byte stores for the partial words at its two ends. A lane
// finds the row of an output byte with a cursor over the 33 offsets in shared
// memory (its output positions only grow).
constexpr int kCopyThreads = 256;
constexpr int kCopyUnroll = 4;

__global__ void __launch_bounds__(kCopyThreads)
    csv_copy_strings_kernel(const uint8_t* __restrict__ text, const int64_t* __restrict__ str_start,
                            const int32_t* __restrict__ offs, uint8_t* __restrict__ out, int64_t n) {
  __shared__ int32_t s_off[kCopyThreads / 32][33];
  __shared__ int64_t s_delta[kCopyThreads / 32][32];  // text offset - output offset, per row
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
  const int32_t* off = s_off[wi];
  const int64_t* delta = s_delta[wi];
  const int64_t n_groups = (n + 31) / 32;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t g = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; g < n_groups; g += nw) {
    const int64_t r0 = g * 32;
    const int nr = static_cast<int>(n - r0 < 32 ? n - r0 : 32);
    if (lane < nr) {
      const int32_t o = offs[r0 + lane];
      s_off[wi][lane] = o;
      s_delta[wi][lane] = str_start[r0 + lane] - o;
    }
    if (lane == 0) s_off[wi][nr] = offs[r0 + nr];
    __syncwarp();
    const int32_t o0 = off[0], o1 = off[nr];
    const int32_t w0 = (o0 + 3) >> 2, w1 = o1 >> 2;  // whole output words [w0, w1)
    {
      // partial words: bytes [o0, min(4 w0, o1)) and [max(4 w1, 4 w0), o1), three at most each
      const int32_t head_end = 4 * w0 < o1 ? 4 * w0 : o1;
      const int32_t tail_beg = 4 * w1 > 4 * w0 ? 4 * w1 : 4 * w0;
      int32_t q = -1;
      if (lane < 4 && o0 + lane < head_end) q = o0 + lane;
      if (lane >= 4 && lane < 8 && tail_beg + lane - 4 < o1) q = tail_beg + lane - 4;
      if (q >= 0) {
        int row = 0;
        while (off[row + 1] <= q) ++row;  // bounded: q < o1 = off[nr]
        out[q] = text[delta[row] + q];
      }
    }
    int row = 0;
    int32_t row_end = off[1];
    int64_t d = delta[0];
    for (int32_t wd = w0 + lane; wd < w1; wd += 32 * kCopyUnroll) {
      uint32_t v[kCopyUnroll];
#pragma unroll
      for (int u = 0; u < kCopyUnroll; ++u) {
        const int32_t word = wd + 32 * u;
        uint32_t x = 0;
        if (word < w1) {
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int32_t q = 4 * word + b;
            while (q >= row_end) {  // bounded: q < o1 = off[nr]
              ++row;
              row_end = off[row + 1];
              d = delta[row];
            }
            x |= static_cast<uint32_t>(text[d + q]) << (8 * b);
          }
        }
        v[u] = x;
      }
#pragma unroll
      for (int u = 0; u < kCopyUnroll; ++u)
        if (wd + 32 * u < w1) reinterpret_cast<uint32_t*>(out)[wd + 32 * u] = v[u];
    }
    __syncwarp();  // the shared offsets are rewritten by the next group
  }
}

}  // namespace

TupleSetPtr csv_parse(const char* device_text, int64_t n_bytes, char delimiter, bool has_header,
                      const std::vector<CsvField>& fields, const std::vector<int>& emit, cudaStream_t s) {
  if (fields.empty()) fail(GFPDB_EINVAL, "CSV schema has no fields");
  if (static_cast<int>(emit.size()) > kCsvMaxOut) fail(GFPDB_EUNSUPPORTED, "too many CSV columns to emit");
  if (static_cast<int>(fields.size()) > 256) fail(GFPDB_EUNSUPPORTED, "too many CSV fields per line");
  if (n_bytes >= (int64_t{1} << 40)) fail(GFPDB_EUNSUPPORTED, "CSV text too large");
  const uint8_t* text = reinterpret_cast<const uint8_t*>(device_text);
  if ((reinterpret_cast<uintptr_t>(text) & 15u) != 0) fail(GFPDB_EINVAL, "CSV text must be 16-byte aligned");

  if (static_cast<int>(fields.size()) > kCsvMaxFields) fail(GFPDB_EUNSUPPORTED, "too many CSV fields per line");
  const int F = static_cast<int>(fields.size());
  // (1)-(2): separators per tile, their scans, the total
  const int64_t n_tiles = n_bytes > 0 ? (n_bytes + kCsvTile - 1) / kCsvTile : 0;
  auto tiles = make_buffer(std::max<int64_t>(n_tiles, 1) * 16 + 16, s);
  auto masks = make_buffer(std::max<int64_t>(n_tiles, 1) * kCsvThreads * 8, s);  // one word per chunk of every tile
  int64_t* tile_count = tiles->as<int64_t>();
  int64_t* tile_last = tile_count + std::max<int64_t>(n_tiles, 1);
  int64_t* tot = tile_last + std::max<int64_t>(n_tiles, 1);
  int64_t host_tot[2] = {0, '\n'};
  if (n_tiles > 0) {
    if (n_tiles >= INT32_MAX) fail(GFPDB_EUNSUPPORTED, "CSV text too large");
    {
      ProfScope prof("csv_index_kernel", s);
      csv_index_kernel<<<static_cast<int>(n_tiles), kCsvThreads, 0, s>>>(text, n_bytes, static_cast<uint8_t>(delimiter),
                                                                        tile_count, tile_last, masks->as<uint64_t>());
      after_launch("csv_index_kernel");
      prof.stop(static_cast<double>(n_bytes));
    }
    csv_tile_scan_kernel<<<1, kCsvScanThreads, 0, s>>>(tile_count, tile_last, n_tiles, text, n_bytes, tot);
    after_launch("csv_tile_scan_kernel");
    GF_CUDA(cudaMemcpyAsync(host_tot, tot, sizeof(host_tot), cudaMemcpyDeviceToHost, s));
    sync(s);
  }
  const bool virtual_end = n_bytes > 0 && host_tot[1] != '\n';
  const int64_t seps = host_tot[0] + (virtual_end ? 1 : 0);
  if (seps % F != 0)
    fail(GFPDB_EINVAL, "malformed CSV field or wrong field count near data row " + std::to_string(seps / F));
  const int64_t lines = seps / F;
  const int64_t skip = has_header && lines > 0 ? 1 : 0;
  const int64_t n_rows = lines - skip;

  // (3) fields
  std::vector<Field> out_fields;
  std::vector<BufferPtr> bufs(emit.size()), sstart(emit.size());
  CsvParams* pp = new CsvParams;
  std::unique_ptr<CsvParams> holder(pp);
  CsvParams& p = *pp;
  std::memset(&p, 0, sizeof(p));
  p.text = text;
  p.n = n_bytes;
  p.tile_base = tile_count;
  p.tile_prev = tile_last;
  p.chunk_masks = masks->as<uint64_t>();
  p.n_rows = n_rows;
  p.n_fields = F;
  p.header = static_cast<int32_t>(skip);
  p.virtual_end = virtual_end ? 1 : 0;
  p.delim = static_cast<uint8_t>(delimiter);
  for (int i = 0; i < kCsvMaxFields; ++i) p.slot[i] = -1;
  auto status = make_filled(sizeof(DevStatus), 0, s);
  p.st = status->as<DevStatus>();
  for (size_t k = 0; k < emit.size(); ++k) {
    const CsvField& f = fields[emit[k]];
    if (p.slot[emit[k]] >= 0) fail(GFPDB_EINVAL, "CSV column '" + f.name + "' projected twice");
    p.slot[emit[k]] = static_cast<int16_t>(k);
    out_fields.push_back(Field{f.name, f.type});
    CsvOut& o = p.out[k];
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
  if (n_tiles > 0) {
    ProfScope prof("csv_fields_kernel", s);
    csv_fields_kernel<<<static_cast<int>(n_tiles), kCsvThreads, 0, s>>>(p);
    after_launch("csv_fields_kernel");
    double out_w = 0;
    for (auto& f : out_fields) out_w += f.type == DType::Utf8 ? 12 : dtype_width(f.type);
    prof.stop(static_cast<double>(n_bytes) + static_cast<double>(n_rows) * out_w);
  }
  // (5) utf8 bytes: every utf8 column's length prefix sum, then one
  // synchronization for the parse status and all their totals (the parse
  // status first: a malformed text reports as such), then the byte copies
  std::vector<size_t> utf8;
  for (size_t k = 0; k < emit.size(); ++k)
    if (out_fields[k].type == DType::Utf8) utf8.push_back(k);
  std::vector<BufferPtr> offs(emit.size()), bytes(emit.size());
  std::vector<int64_t> totals(utf8.size(), 0);
  {
    auto sts = make_filled(static_cast<int64_t>(utf8.size() * sizeof(DevStatus)) + 64, 0, s);
    DevStatus* st = sts->as<DevStatus>();
    for (size_t u = 0; u < utf8.size(); ++u) {
      const size_t k = utf8[u];
      offs[k] = make_buffer((n_rows + 1) * 4, s);
      exclusive_scan_i32_async(bufs[k]->as<int32_t>(), offs[k]->as<int32_t>(), n_rows, st + u, s);
    }
    std::vector<DevStatus> hs(utf8.size() + 1);
    GF_CUDA(cudaMemcpyAsync(hs.data(), status->data(), sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
    if (!utf8.empty())
      GF_CUDA(cudaMemcpyAsync(hs.data() + 1, st, utf8.size() * sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
    sync(s);
    if (hs[0].code == GFPDB_EINVAL)
      fail(GFPDB_EINVAL, "malformed CSV field or wrong field count near data row " + std::to_string(hs[0].detail));
    raise_device_status(hs[0], "CSV parse");
    for (size_t u = 0; u < utf8.size(); ++u) {
      raise_device_status(hs[u + 1], "prefix sum");
      if (hs[u + 1].value > INT32_MAX) fail(GFPDB_EUNSUPPORTED, "utf8 column exceeds 2 GiB of bytes");
      totals[u] = hs[u + 1].value;
    }
  }
  for (size_t u = 0; u < utf8.size(); ++u) {
    const size_t k = utf8[u];
    const int64_t total = totals[u];
    bytes[k] = make_buffer(total, s);
    if (n_rows > 0 && total > 0) {
      const int64_t groups = (n_rows + 31) / 32;
      int64_t blocks = (groups + kCopyThreads / 32 - 1) / (kCopyThreads / 32);
      int64_t cap = static_cast<int64_t>(num_sms()) * 16;
      ProfScope prof("csv_copy_strings_kernel", s);
      csv_copy_strings_kernel<<<static_cast<int>(blocks < cap ? blocks : cap), kCopyThreads, 0, s>>>(
          text, sstart[k]->as<int64_t>(), offs[k]->as<int32_t>(), bytes[k]->as<uint8_t>(), n_rows);
      after_launch("csv_copy_strings_kernel");
      prof.stop(2.0 * static_cast<double>(total) + 12.0 * static_cast<double>(n_rows));
    }
  }
  std::vector<ColumnPtr> cols;
  for (size_t k = 0; k < emit.size(); ++k)
    cols.push_back(out_fields[k].type == DType::Utf8 ? make_utf8_column(n_rows, offs[k], bytes[k])
                                                     : make_fixed_column(out_fields[k].type, n_rows, bufs[k]));
  return TupleSet::make(std::move(out_fields), std::move(cols), n_rows);
}

}  // namespace gfpdb
