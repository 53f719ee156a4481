// Parquet column decoding on the device: the data half of Arrow's
// parquet::arrow::FileReader::ReadTable that ParquetReader::readImpl drives
// (fpdb-tuple/src/parquet/ParquetReader.cpp:12-42), after the host has read
// the footer and page headers (host/parquet_meta.cpp). The page formats are
// the public Apache Parquet specification's: PLAIN values (little-endian
// fixed width; byte arrays as a 4-byte length then the bytes), dictionary
// pages (PLAIN) with data pages of RLE / bit-packed hybrid indices behind a
// bit-width byte, definition levels of optional columns as a 4-byte length
// and an RLE / bit-packed hybrid run (v1) or a separate uncompressed prefix
// (v2), and the snappy block format.
//
// Launches:
//   parquet_snappy_kernel  one warp per snappy page: lane 0 reads each
//                          element's tag (literal, or a copy with a 1-, 2- or
//                          4-byte offset) and the warp moves its bytes, 32 at
//                          a time (copies whose source overlaps their output
//                          go in steps of the offset);
//   parquet_pages_kernel   one CTA per page: thread 0 skips (and checks) the
//                          definition levels, walks byte-array lengths (data
//                          and dictionary pages) and reads the dictionary
//                          indices' run headers, up to 256 a round, and every
//                          thread then decodes the round's indices, a
//                          fixed-width column's straight into its values;
//   parquet_values_kernel  per plain data page and value: fixed-width values
//                          copied into the output column; byte arrays (plain
//                          or dictionary-encoded) get their source and
//                          length;
//   then per utf8 column a prefix sum of the lengths and a byte copy.
#include <cstring>
#include <vector>

#include "../host/parquet_meta.h"
#include "common.cuh"
#include "launch.h"

namespace gfpdb {
namespace {

struct PageDev {
  const uint8_t* body;    // page body on the device (after its header)
  uint8_t* inflated;      // snappy pages: the decompressed body (v2: the values part)
  const uint8_t* values;  // set by parquet_pages_kernel: the first value byte
  int32_t body_len;
  int32_t inflated_len;
  int32_t values_len;     // set with `values`
  int32_t type;           // PageType
  int32_t encoding;
  int32_t snappy;         // 1: the values live in `inflated`
  int32_t num_values;
  int32_t v2_levels;      // data page v2: level bytes ahead of the values
  int32_t v1_def;         // data page v1 of an optional column
  int32_t width;          // fixed-width bytes, 0 for byte arrays
  int32_t dict_page;      // data pages: their dictionary page's index, -1
  int32_t pad;
  int64_t first_row;
  int64_t dict_base;      // byte-array dictionary pages: first entry in dict_ptr / dict_len
  int32_t* idx;           // dictionary-encoded columns: per-row entry
  uint64_t* row_ptr;      // byte-array columns: per-row value address
  int32_t* row_len;       //   and length
  uint8_t* fixed_out;     // fixed-width columns: the output values
};

struct DictArrays {
  uint64_t* ptr;  // byte-array dictionary entries: address
  int32_t* len;   //   and length
};

__device__ __forceinline__ uint32_t le32(const uint8_t* p) {
  return static_cast<uint32_t>(p[0]) | (static_cast<uint32_t>(p[1]) << 8) | (static_cast<uint32_t>(p[2]) << 16) |
         (static_cast<uint32_t>(p[3]) << 24);
}

// Snappy block format: a varint of the uncompressed length, then elements.
__device__ void snappy_warp(const uint8_t* src, int32_t n, uint8_t* dst, int32_t cap, DevStatus* st, int page) {
  const int lane = threadIdx.x & 31;
  int32_t ip = 0;
  int ok = 1;
  if (lane == 0) {
    uint32_t ulen = 0;
    int shift = 0;
    ok = 0;
    while (ip < n && shift <= 28) {
      const uint8_t b = src[ip++];
      ulen |= static_cast<uint32_t>(b & 0x7f) << shift;
      if (!(b & 0x80)) {
        ok = ulen == static_cast<uint32_t>(cap) ? 1 : 0;
        break;
      }
      shift += 7;
    }
  }
  ok = __shfl_sync(0xffffffffu, ok, 0);
  if (!ok) {
    if (lane == 0) raise_status(st, GFPDB_EINVAL, 100000 + page);
    return;
  }
  int32_t op = 0;
  for (;;) {
    int32_t kind = 0, len = 0, off = 0, lit = 0;
    if (lane == 0) {
      if (ip >= n) {
        kind = -1;
      } else {
        const uint8_t tag = src[ip++];
        const int t = tag & 3;
        if (t == 0) {
          len = (tag >> 2) + 1;
          if (len > 60) {
            const int nb = len - 60;
            len = 0;
            if (ip + nb > n) {
              kind = -2;
            } else {
              for (int k = 0; k < nb; ++k) len |= static_cast<int32_t>(src[ip + k]) << (8 * k);
              ip += nb;
              len += 1;
            }
          }
          lit = ip;
          ip += len;
          if (kind == 0) kind = (len <= 0 || ip > n) ? -2 : 1;
        } else {
          const int nb = t == 1 ? 1 : (t == 2 ? 2 : 4);
          if (ip + nb > n) {
            kind = -2;
          } else {
            if (t == 1) {
              len = 4 + ((tag >> 2) & 7);
              off = ((tag >> 5) << 8) | src[ip];
            } else {
              len = 1 + (tag >> 2);
              off = t == 2 ? (src[ip] | (src[ip + 1] << 8)) : static_cast<int32_t>(le32(src + ip));
            }
            ip += nb;
            kind = (off <= 0 || off > op) ? -2 : 2;
          }
        }
        if (kind > 0 && (len > cap - op)) kind = -2;
      }
    }
    kind = __shfl_sync(0xffffffffu, kind, 0);
    if (kind < 0) {
      if (kind == -2 && lane == 0) raise_status(st, GFPDB_EINVAL, 100000 + page);
      break;
    }
    len = __shfl_sync(0xffffffffu, len, 0);
    off = __shfl_sync(0xffffffffu, off, 0);
    lit = __shfl_sync(0xffffffffu, lit, 0);
    if (kind == 1) {
      for (int32_t i = lane; i < len; i += 32) dst[op + i] = src[lit + i];
    } else {
      const int32_t step = off < 32 ? off : 32;  // a step never reads what it writes
      for (int32_t base = 0; base < len; base += step) {
        const int32_t i = base + lane;
        if (lane < step && i < len) dst[op + i] = dst[op + i - off];
        __syncwarp();
      }
    }
    __syncwarp();
    op += len;
  }
  if (lane == 0 && op != cap) raise_status(st, GFPDB_EINVAL, 100000 + page);
}

__global__ void __launch_bounds__(256) parquet_snappy_kernel(PageDev* pages, const int32_t* list, int32_t n,
                                                             DevStatus* st) {
  const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int64_t warps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t w = warp; w < n; w += warps) {
    __syncwarp();
    const int p = list[w];
    const PageDev& pg = pages[p];
    const int32_t skip = pg.type == parquet::PAGE_DATA_V2 ? pg.v2_levels : 0;
    snappy_warp(pg.body + skip, pg.body_len - skip, pg.inflated, pg.inflated_len, st, p);
  }
}

// One run header of an RLE / bit-packed hybrid stream at p[*at]: returns
// false past the end.
__device__ __forceinline__ bool run_header(const uint8_t* p, int32_t n, int32_t* at, uint32_t* h) {
  uint32_t v = 0;
  for (int shift = 0; shift <= 28; shift += 7) {
    if (*at >= n) return false;
    const uint8_t b = p[(*at)++];
    v |= static_cast<uint32_t>(b & 0x7f) << shift;
    if (!(b & 0x80)) {
      *h = v;
      return true;
    }
  }
  return false;
}

__device__ __forceinline__ void copy_value(const uint8_t* src, uint8_t* dst, int w) {
  if (w == 8 && !(reinterpret_cast<uintptr_t>(src) & 7)) {
    *reinterpret_cast<uint64_t*>(dst) = *reinterpret_cast<const uint64_t*>(src);
  } else if (w == 4 && !(reinterpret_cast<uintptr_t>(src) & 3)) {
    *reinterpret_cast<uint32_t*>(dst) = *reinterpret_cast<const uint32_t*>(src);
  } else {
    for (int k = 0; k < w; ++k) dst[k] = src[k];
  }
}

constexpr int kPqThreads = 256;
constexpr int kPqRuns = 256;  // run headers read per round

// One CTA per page. Thread 0 does the sequential parts (definition levels,
// byte-array lengths, run headers); the dictionary indices of each round of
// up to kPqRuns runs are then decoded by every thread, a value finding its
// run by binary search over the runs' first values. A fixed-width column's
// index is looked up in its dictionary page at once and the value written
// to the output column (the dictionary page's body is read as the host laid
// it out, not through fields another CTA of this launch sets); a byte-array
// column's index is kept for parquet_values_kernel, which runs after the
// dictionary pages' entries are known.
__global__ void __launch_bounds__(kPqThreads) parquet_pages_kernel(PageDev* pages, int32_t n_pages, DictArrays dicts,
                                                                   DevStatus* st) {
  __shared__ int32_t s_first[kPqRuns + 1];  // the page value index each run starts at; then the round's end
  __shared__ int32_t s_start[kPqRuns];      // bit-packed runs: first byte; RLE runs: -1
  __shared__ uint32_t s_value[kPqRuns];     // RLE runs: the value
  __shared__ int32_t s_n, s_ok, s_at, s_done, s_bw;
  for (int64_t w = blockIdx.x; w < n_pages; w += gridDim.x) {
    __syncthreads();  // the previous page's shared state is no longer read
    PageDev& pg = pages[w];
    const uint8_t* base;
    int32_t blen;
    if (pg.snappy) {
      base = pg.inflated;
      blen = pg.inflated_len;
    } else {
      const int32_t skip = pg.type == parquet::PAGE_DATA_V2 ? pg.v2_levels : 0;
      base = pg.body + skip;
      blen = pg.body_len - skip;
    }
    if (threadIdx.x == 0) {
      int ok = 1;
      if (pg.v1_def) {  // 4-byte length, then the levels: every one must be 1 (no nulls)
        ok = 0;
        if (blen >= 4) {
          const int32_t len = static_cast<int32_t>(le32(base));
          if (len >= 0 && len <= blen - 4) {
            const uint8_t* lv = base + 4;
            int32_t at = 0, seen = 0;
            ok = 1;
            while (seen < pg.num_values && ok) {
              uint32_t h;
              if (!run_header(lv, len, &at, &h)) {
                ok = 0;
                break;
              }
              if (h & 1) {  // bit-packed: (h >> 1) groups of 8 one-bit levels
                const int32_t bytes = static_cast<int32_t>(h >> 1);
                if (bytes > len - at) {
                  ok = 0;
                  break;
                }
                for (int32_t b = 0; b < bytes && ok; ++b) {
                  const int32_t valid = pg.num_values - seen - 8 * b;
                  const uint32_t need = valid >= 8 ? 0xffu : ((1u << (valid > 0 ? valid : 0)) - 1u);
                  if ((lv[at + b] & need) != need) ok = 0;  // a 0 level: a null
                }
                at += bytes;
                seen += 8 * bytes;
              } else {  // RLE: (h >> 1) copies of a one-byte level
                if (at >= len || lv[at] != 1) {
                  ok = 0;
                  break;
                }
                ++at;
                seen += static_cast<int32_t>(h >> 1);
              }
            }
            base += 4 + len;
            blen -= 4 + len;
          }
        }
        if (!ok) raise_status(st, GFPDB_EUNSUPPORTED, 200000 + static_cast<int32_t>(w));  // nulls, or bad levels
      }
      if (ok) {
        pg.values = base;
        pg.values_len = blen;
        const bool bytes_walk = pg.width == 0 && (pg.type == parquet::PAGE_DICTIONARY || pg.encoding == parquet::ENC_PLAIN);
        if (bytes_walk) {  // byte arrays: each value's address and length
          const bool dict = pg.type == parquet::PAGE_DICTIONARY;
          int32_t at = 0;
          for (int32_t e = 0; e < pg.num_values; ++e) {
            int32_t len = -1;
            if (blen - at >= 4) {
              len = static_cast<int32_t>(le32(base + at));
              at += 4;
            }
            if (len < 0 || len > blen - at) {
              raise_status(st, GFPDB_EINVAL, (dict ? 300000 : 400000) + static_cast<int32_t>(w));
              ok = 0;
              break;
            }
            if (dict) {
              dicts.ptr[pg.dict_base + e] = reinterpret_cast<uint64_t>(base + at);
              dicts.len[pg.dict_base + e] = len;
            } else {
              pg.row_ptr[pg.first_row + e] = reinterpret_cast<uint64_t>(base + at);
              pg.row_len[pg.first_row + e] = len;
            }
            at += len;
          }
        } else if (pg.width > 0 && (pg.type == parquet::PAGE_DICTIONARY || pg.encoding == parquet::ENC_PLAIN) &&
                   static_cast<int64_t>(pg.num_values) * pg.width > blen) {
          raise_status(st, GFPDB_EINVAL, 400000 + static_cast<int32_t>(w));
          ok = 0;
        }
      }
      const bool indices = ok && pg.type != parquet::PAGE_DICTIONARY && pg.encoding != parquet::ENC_PLAIN;
      s_bw = blen > 0 ? base[0] : 99;
      if (indices && (s_bw > 32 || pg.dict_page < 0 || pg.dict_page >= n_pages)) {
        raise_status(st, GFPDB_EINVAL, 500000 + static_cast<int32_t>(w));
        ok = 0;
      }
      s_ok = indices ? ok : 0;
      s_at = 1;
      s_done = 0;
    }
    __syncthreads();
    if (!s_ok) continue;
    // Dictionary indices: a bit-width byte, then RLE / bit-packed hybrid runs.
    base = pg.values;
    blen = pg.values_len;
    const int32_t bw = s_bw;
    const uint64_t mask = bw == 32 ? 0xffffffffull : ((1ull << bw) - 1ull);
    // a fixed-width column's dictionary: its page's values as laid out on
    // the host (dictionary pages carry no levels), its entry count and bytes
    const uint8_t* dvals = nullptr;
    int64_t dlen = 0;
    int32_t dn = 0;
    if (pg.width > 0) {
      const PageDev& dp = pages[pg.dict_page];
      dvals = dp.snappy ? dp.inflated : dp.body;
      dlen = dp.snappy ? dp.inflated_len : dp.body_len;
      dn = dp.num_values;
    }
    for (;;) {
      if (threadIdx.x == 0) {
        int32_t n = 0, at = s_at, done = s_done;
        while (n < kPqRuns && done < pg.num_values) {
          uint32_t h;
          if (!run_header(base, blen, &at, &h)) {
            s_ok = 0;
            break;
          }
          int64_t count;
          if (h & 1) {
            const int64_t groups = h >> 1;
            if (groups * bw > blen - at) {
              s_ok = 0;
              break;
            }
            s_start[n] = at;
            at += static_cast<int32_t>(groups * bw);
            count = groups * 8;
          } else {
            const int32_t vb = (bw + 7) / 8;
            if (vb > blen - at) {
              s_ok = 0;
              break;
            }
            uint32_t v = 0;
            for (int k = 0; k < vb; ++k) v |= static_cast<uint32_t>(base[at + k]) << (8 * k);
            at += vb;
            s_start[n] = -1;
            s_value[n] = v;
            count = h >> 1;
          }
          if (count <= 0) {
            s_ok = 0;
            break;
          }
          s_first[n] = done;
          done += static_cast<int32_t>(count < pg.num_values - done ? count : pg.num_values - done);
          ++n;
        }
        s_first[n] = done;
        s_n = s_ok ? n : 0;
        s_at = at;
        s_done = done;
        if (!s_ok) raise_status(st, GFPDB_EINVAL, 500000 + static_cast<int32_t>(w));
      }
      __syncthreads();
      const int32_t n = s_n;
      if (n == 0) break;
      const int32_t v0 = s_first[0], v1 = s_first[n];
      // unrolled so that several values' loads are in flight together
#pragma unroll 4
      for (int32_t v = v0 + static_cast<int32_t>(threadIdx.x); v < v1; v += kPqThreads) {
        int32_t lo = 0, hi = n - 1;  // the run holding v: the last with s_first <= v
        while (lo < hi) {
          const int32_t mid = (lo + hi + 1) >> 1;
          if (s_first[mid] <= v) lo = mid;
          else hi = mid - 1;
        }
        uint32_t idx;
        if (s_start[lo] < 0) {
          idx = s_value[lo];
        } else {
          const int64_t bit = static_cast<int64_t>(v - s_first[lo]) * bw;
          const uint8_t* q = base + s_start[lo] + (bit >> 3);
          uint64_t x = 0;
          const int nb = (static_cast<int>(bit & 7) + bw + 7) / 8;  // bytes the value spans (within the run)
          for (int k = 0; k < nb; ++k) x |= static_cast<uint64_t>(__ldg(q + k)) << (8 * k);
          idx = static_cast<uint32_t>((x >> (bit & 7)) & mask);
        }
        if (pg.width > 0) {
          if (idx >= static_cast<uint32_t>(dn) || (static_cast<int64_t>(idx) + 1) * pg.width > dlen) {
            raise_status(st, GFPDB_EINVAL, 600000 + static_cast<int32_t>(w));
            continue;
          }
          // the value's 4-byte words from the two aligned words around each
          // (the arena and the inflated buffer carry 16 bytes of tail padding)
          const uint8_t* sp = dvals + static_cast<int64_t>(idx) * pg.width;
          const uint32_t* al = reinterpret_cast<const uint32_t*>(reinterpret_cast<uintptr_t>(sp) & ~uintptr_t{3});
          const uint32_t sh = 8u * static_cast<uint32_t>(reinterpret_cast<uintptr_t>(sp) & 3u);
          uint32_t* dw = reinterpret_cast<uint32_t*>(pg.fixed_out + (pg.first_row + v) * pg.width);
          for (int k = 0; k < pg.width / 4; ++k) dw[k] = __funnelshift_r(__ldg(al + k), __ldg(al + k + 1), sh);
        } else {
          pg.idx[pg.first_row + v] = static_cast<int32_t>(idx);
        }
      }
      const bool more = s_done < pg.num_values;
      __syncthreads();  // the runs are read before thread 0 rewrites them
      if (!more) break;
    }
  }
}

// blockIdx.y: a data page (index into `list`); values over x.
__global__ void __launch_bounds__(256) parquet_values_kernel(const PageDev* pages, const int32_t* list, DictArrays dicts,
                                                             DevStatus* st) {
  const PageDev& pg = pages[list[blockIdx.y]];
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  const bool dict = pg.encoding != parquet::ENC_PLAIN;
  const PageDev* dp = dict ? &pages[pg.dict_page] : nullptr;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < pg.num_values; i += stride) {
    const int64_t row = pg.first_row + i;
    if (pg.width > 0) {
      // bounds: a page whose levels or sizes were bad has values_len 0
      // plain values only: a fixed-width dictionary page is decoded to its
      // values by the page pass and never listed here
      if (dict || (i + 1) * pg.width > pg.values_len) {
        raise_status(st, GFPDB_EINVAL, 600000 + static_cast<int32_t>(blockIdx.y));
        continue;
      }
      // the value's 4-byte words from the two aligned words around each
      // (the arena and the inflated buffer carry 16 bytes of tail padding)
      const uint8_t* sp = pg.values + i * pg.width;
      const uint32_t* al = reinterpret_cast<const uint32_t*>(reinterpret_cast<uintptr_t>(sp) & ~uintptr_t{3});
      const uint32_t sh = 8u * static_cast<uint32_t>(reinterpret_cast<uintptr_t>(sp) & 3u);
      uint32_t* dw = reinterpret_cast<uint32_t*>(pg.fixed_out + row * pg.width);
      for (int k = 0; k < pg.width / 4; ++k) dw[k] = __funnelshift_r(al[k], al[k + 1], sh);
    } else if (dict) {
      const int32_t e = pg.idx[row];
      if (e < 0 || e >= dp->num_values) {
        raise_status(st, GFPDB_EINVAL, 600000 + static_cast<int32_t>(blockIdx.y));
        pg.row_ptr[row] = 0;
        pg.row_len[row] = 0;
        continue;
      }
      pg.row_ptr[row] = dicts.ptr[dp->dict_base + e];
      pg.row_len[row] = dicts.len[dp->dict_base + e];
    }
  }
}

__global__ void parquet_bytes_kernel(const uint64_t* __restrict__ ptr, const int32_t* __restrict__ offs, int64_t n,
                                     uint8_t* __restrict__ out) {
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
    const uint8_t* src = reinterpret_cast<const uint8_t*>(ptr[r]);
    const int32_t o = offs[r], len = offs[r + 1] - o;
    for (int32_t k = 0; k < len; ++k) out[o + k] = src[k];
  }
}

int grid_parquet(int64_t n) {
  int64_t b = (n + 255) / 256;
  const int64_t cap = static_cast<int64_t>(num_sms()) * 8;
  if (b > cap) b = cap;
  return static_cast<int>(b < 1 ? 1 : b);
}

}  // namespace

TupleSetPtr parquet_read(const uint8_t* file, int64_t size, const std::vector<std::string>& names, int64_t start_pos,
                         int64_t end_pos, cudaStream_t s) {
  const parquet::Layout L = parquet::read_layout(file, size, names, start_pos, end_pos);
  const int64_t rows = L.num_rows;
  if (rows > INT32_MAX) fail(GFPDB_EUNSUPPORTED, "a Parquet read of more than 2^31 - 1 rows");
  const int nc = static_cast<int>(L.columns.size());

  // the column chunks' bytes on the device, one copy each
  std::vector<int64_t> chunk_at(L.chunks.size());
  int64_t arena_bytes = 0;
  for (size_t c = 0; c < L.chunks.size(); ++c) {
    chunk_at[c] = arena_bytes;
    arena_bytes += (L.chunks[c].end - L.chunks[c].begin + 15) / 16 * 16;
  }
  auto arena = make_buffer(arena_bytes + 16, s);  // tail padding: 4-byte word reads past a value's end
  for (size_t c = 0; c < L.chunks.size(); ++c)
    copy_h2d(arena->as<uint8_t>() + chunk_at[c], file + L.chunks[c].begin, L.chunks[c].end - L.chunks[c].begin, s);

  // per-column outputs and working arrays
  std::vector<BufferPtr> fixed(nc), row_ptr(nc), row_len(nc), idx(nc);
  std::vector<bool> has_dict(nc, false);
  for (const auto& pg : L.pages)
    if (pg.type != parquet::PAGE_DICTIONARY && pg.encoding != parquet::ENC_PLAIN) has_dict[pg.column] = true;
  for (int c = 0; c < nc; ++c) {
    const DType t = L.columns[c].dtype;
    if (t == DType::Utf8) {
      row_ptr[c] = make_buffer((rows > 0 ? rows : 1) * 8, s);
      row_len[c] = make_buffer((rows > 0 ? rows : 1) * 4, s);
    } else {
      fixed[c] = make_buffer((rows > 0 ? rows : 1) * dtype_width(t), s);
    }
    if (has_dict[c] && t == DType::Utf8) idx[c] = make_buffer((rows > 0 ? rows : 1) * 4, s);
  }

  // page descriptors
  std::vector<PageDev> pd(L.pages.size());
  std::vector<int32_t> snappy_list, data_list;
  int64_t inflate_bytes = 0, dict_entries = 0;
  std::vector<int64_t> inflate_at(L.pages.size(), -1);
  for (size_t p = 0; p < L.pages.size(); ++p) {
    const auto& pg = L.pages[p];
    const bool v2 = pg.type == parquet::PAGE_DATA_V2;
    const bool snappy = pg.codec == parquet::CODEC_SNAPPY && !(v2 && !pg.v2_compressed);
    if (snappy) {
      inflate_at[p] = inflate_bytes;
      inflate_bytes += (static_cast<int64_t>(pg.uncompressed) - (v2 ? pg.v2_levels : 0) + 15) / 16 * 16;
      snappy_list.push_back(static_cast<int32_t>(p));
    } else if ((v2 ? pg.compressed - pg.v2_levels : pg.compressed) !=
               (v2 ? pg.uncompressed - pg.v2_levels : pg.uncompressed)) {
      fail(GFPDB_EINVAL, "Parquet uncompressed page sizes disagree");
    }
    // data pages the values pass reads: plain pages, and dictionary-encoded
    // byte-array pages (a fixed-width column's dictionary indices become
    // values in the page pass)
    const bool fixed_dict = L.columns[pg.column].dtype != DType::Utf8 && pg.encoding != parquet::ENC_PLAIN;
    if (pg.type != parquet::PAGE_DICTIONARY && !fixed_dict) data_list.push_back(static_cast<int32_t>(p));
  }
  auto inflated = make_buffer(inflate_bytes + 16, s);
  for (size_t p = 0; p < L.pages.size(); ++p) {
    const auto& pg = L.pages[p];
    const int c = pg.column;
    const bool v2 = pg.type == parquet::PAGE_DATA_V2;
    PageDev& d = pd[p];
    std::memset(&d, 0, sizeof(d));
    d.body = arena->as<uint8_t>() + chunk_at[pg.chunk] + (pg.data_offset - L.chunks[pg.chunk].begin);
    d.body_len = pg.compressed;
    d.snappy = inflate_at[p] >= 0 ? 1 : 0;
    d.inflated = d.snappy ? inflated->as<uint8_t>() + inflate_at[p] : nullptr;
    d.inflated_len = d.snappy ? pg.uncompressed - (v2 ? pg.v2_levels : 0) : 0;
    d.type = pg.type;
    d.encoding = pg.encoding;
    d.num_values = pg.num_values;
    d.v2_levels = pg.v2_levels;
    d.v1_def = pg.v1_def_levels ? 1 : 0;
    d.width = L.columns[c].dtype == DType::Utf8 ? 0 : dtype_width(L.columns[c].dtype);
    d.dict_page = pg.dict_page;
    d.first_row = pg.first_row;
    if (pg.type == parquet::PAGE_DICTIONARY && d.width == 0) {
      d.dict_base = dict_entries;
      dict_entries += pg.num_values;
    }
    d.idx = idx[c] ? idx[c]->as<int32_t>() : nullptr;
    d.row_ptr = row_ptr[c] ? row_ptr[c]->as<uint64_t>() : nullptr;
    d.row_len = row_len[c] ? row_len[c]->as<int32_t>() : nullptr;
    d.fixed_out = fixed[c] ? fixed[c]->as<uint8_t>() : nullptr;
  }
  DictArrays dicts{};
  BufferPtr dict_ptr, dict_len;
  if (dict_entries > 0) {
    dict_ptr = make_buffer(dict_entries * 8, s);
    dict_len = make_buffer(dict_entries * 4, s);
    dicts.ptr = dict_ptr->as<uint64_t>();
    dicts.len = dict_len->as<int32_t>();
  }
  auto status = make_filled(sizeof(DevStatus), 0, s);
  DevStatus* st = status->as<DevStatus>();
  const int64_t np = static_cast<int64_t>(pd.size());
  auto pages_dev = make_buffer((np > 0 ? np : 1) * static_cast<int64_t>(sizeof(PageDev)), s);
  const int64_t nl = static_cast<int64_t>(snappy_list.size() + data_list.size());
  auto lists = make_buffer((nl > 0 ? nl : 1) * 4, s);
  std::vector<int32_t> both(snappy_list);
  both.insert(both.end(), data_list.begin(), data_list.end());
  if (np > 0) GF_CUDA(cudaMemcpyAsync(pages_dev->data(), pd.data(), np * sizeof(PageDev), cudaMemcpyHostToDevice, s));
  if (nl > 0) GF_CUDA(cudaMemcpyAsync(lists->data(), both.data(), nl * 4, cudaMemcpyHostToDevice, s));
  PageDev* pages = pages_dev->as<PageDev>();
  const int32_t* snappy_dev = lists->as<int32_t>();
  const int32_t* data_dev = lists->as<int32_t>() + snappy_list.size();

  if (!snappy_list.empty()) {
    ProfScope prof("parquet_snappy_kernel", s);
    parquet_snappy_kernel<<<grid_parquet(static_cast<int64_t>(snappy_list.size()) * 32), 256, 0, s>>>(
        pages, snappy_dev, static_cast<int32_t>(snappy_list.size()), st);
    after_launch("parquet_snappy_kernel");
    prof.stop(static_cast<double>(inflate_bytes));
  }
  if (np > 0) {
    ProfScope prof("parquet_pages_kernel", s);
    const int64_t most = static_cast<int64_t>(num_sms()) * 8;
    parquet_pages_kernel<<<static_cast<int>(np < most ? np : most), kPqThreads, 0, s>>>(
        pages, static_cast<int32_t>(np), dicts, st);
    after_launch("parquet_pages_kernel");
    prof.stop(0.0);
  }
  if (!data_list.empty()) {
    // each data page's values over up to 64 blocks of 256 threads
    int64_t most = 0;
    for (int32_t p : data_list) most = std::max<int64_t>(most, L.pages[p].num_values);
    const int gx = static_cast<int>(std::min<int64_t>(64, std::max<int64_t>(1, (most + 255) / 256)));
    for (size_t at = 0; at < data_list.size(); at += 65535) {  // grid y limit
      const int gy = static_cast<int>(std::min<size_t>(65535, data_list.size() - at));
      ProfScope prof("parquet_values_kernel", s);
      parquet_values_kernel<<<dim3(gx, gy), 256, 0, s>>>(pages, data_dev + at, dicts, st);
      after_launch("parquet_values_kernel");
      prof.stop(0.0);
    }
  }
  DevStatus h;
  GF_CUDA(cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, s));
  sync(s);
  if (h.code != 0)
    fail(h.code, std::string(h.code == GFPDB_EUNSUPPORTED ? "Parquet column with nulls (definition levels)"
                                                         : "malformed Parquet page data") +
                     " (page " + std::to_string(h.detail % 100000) + ")");

  std::vector<Field> fields;
  std::vector<ColumnPtr> cols;
  for (int c = 0; c < nc; ++c) {
    const DType t = L.columns[c].dtype;
    fields.push_back(Field{L.columns[c].name, t});
    if (t != DType::Utf8) {
      cols.push_back(make_fixed_column(t, rows, fixed[c]));
      continue;
    }
    auto offs = make_buffer((rows + 1) * 4, s);
    const int64_t total = rows > 0 ? exclusive_scan_i32(row_len[c]->as<int32_t>(), offs->as<int32_t>(), rows, s) : 0;
    if (rows == 0) GF_CUDA(cudaMemsetAsync(offs->data(), 0, 4, s));
    auto bytes = make_buffer(total > 0 ? total : 1, s);
    if (total > 0) {
      ProfScope prof("parquet_bytes_kernel", s);
      parquet_bytes_kernel<<<grid_parquet(rows), 256, 0, s>>>(row_ptr[c]->as<uint64_t>(), offs->as<int32_t>(), rows,
                                                              bytes->as<uint8_t>());
      after_launch("parquet_bytes_kernel");
      prof.stop(2.0 * static_cast<double>(total));
    }
    cols.push_back(make_utf8_column(rows, offs, bytes));
  }
  sync(s);  // the page descriptors (host vector) and the arena are released on return
  return TupleSet::make(std::move(fields), std::move(cols), rows);
}

}  // namespace gfpdb
