#include "parquet_meta.h"

#include <algorithm>
#include <cstring>

#include "runtime.h"

namespace gfpdb::parquet {

namespace {

// Well-formed UTF-8 (RFC 3629): no overlong forms, surrogates or code points
// past U+10FFFF.
bool valid_utf8(const std::string& s) {
  const auto* p = reinterpret_cast<const unsigned char*>(s.data());
  const size_t n = s.size();
  for (size_t i = 0; i < n;) {
    const unsigned c = p[i];
    int len;
    unsigned cp;
    if (c < 0x80) {
      ++i;
      continue;
    } else if ((c & 0xE0) == 0xC0) {
      len = 2;
      cp = c & 0x1F;
    } else if ((c & 0xF0) == 0xE0) {
      len = 3;
      cp = c & 0x0F;
    } else if ((c & 0xF8) == 0xF0) {
      len = 4;
      cp = c & 0x07;
    } else {
      return false;
    }
    if (i + static_cast<size_t>(len) > n) return false;
    for (int k = 1; k < len; ++k) {
      if ((p[i + k] & 0xC0) != 0x80) return false;
      cp = (cp << 6) | (p[i + k] & 0x3F);
    }
    if ((len == 2 && cp < 0x80) || (len == 3 && cp < 0x800) || (len == 4 && cp < 0x10000) || cp > 0x10FFFF ||
        (cp >= 0xD800 && cp <= 0xDFFF))
      return false;
    i += static_cast<size_t>(len);
  }
  return true;
}

// Thrift compact protocol (the encoding of Parquet's metadata): field
// headers carry an id delta and a type nibble, integers are zigzag varints,
// binaries and lists a varint length.
enum CType : int { CT_STOP = 0, CT_TRUE = 1, CT_FALSE = 2, CT_BYTE = 3, CT_I16 = 4, CT_I32 = 5, CT_I64 = 6,
                   CT_DOUBLE = 7, CT_BINARY = 8, CT_LIST = 9, CT_SET = 10, CT_MAP = 11, CT_STRUCT = 12 };

class Reader {
 public:
  Reader(const uint8_t* p, int64_t n) : p_(p), n_(n) {}

  int64_t pos() const { return pos_; }

  uint8_t byte() {
    if (pos_ >= n_) fail(GFPDB_EINVAL, "Parquet metadata ends early");
    return p_[pos_++];
  }
  uint64_t varint() {
    uint64_t v = 0;
    for (int shift = 0; shift < 64; shift += 7) {
      const uint8_t b = byte();
      v |= static_cast<uint64_t>(b & 0x7f) << shift;
      if (!(b & 0x80)) return v;
    }
    fail(GFPDB_EINVAL, "Parquet metadata: malformed varint");
  }
  int64_t zigzag() {
    const uint64_t v = varint();
    return static_cast<int64_t>(v >> 1) ^ -static_cast<int64_t>(v & 1);
  }
  std::string binary() {
    const uint64_t len = varint();
    if (len > static_cast<uint64_t>(n_ - pos_)) fail(GFPDB_EINVAL, "Parquet metadata: string runs past the end");
    std::string s(reinterpret_cast<const char*>(p_ + pos_), len);
    pos_ += static_cast<int64_t>(len);
    return s;
  }

  // Next field of a struct: false at its end. *id and *type are set.
  bool field(int16_t* last_id, int* id, int* type) {
    const uint8_t h = byte();
    if (h == CT_STOP) return false;
    *type = h & 0x0f;
    const int delta = h >> 4;
    *id = delta != 0 ? *last_id + delta : static_cast<int>(zigzag());
    *last_id = static_cast<int16_t>(*id);
    return true;
  }
  // List header: element count and type.
  int64_t list(int* elem) {
    const uint8_t h = byte();
    *elem = h & 0x0f;
    const int64_t n = h >> 4;
    return n == 15 ? static_cast<int64_t>(varint()) : n;
  }
  bool boolean(int type) { return type == CT_TRUE; }  // a struct field's value is its type

  // An element of a list, set or map: booleans there are one byte each (in
  // a struct a boolean lives in its field header), so every element consumes
  // input and a corrupt element count runs into the end of the footer.
  void skip_element(int type, int depth) {
    if (type == CT_TRUE || type == CT_FALSE) byte();
    else skip(type, depth);
  }

  void skip(int type, int depth = 0) {
    if (depth > 32) fail(GFPDB_EINVAL, "Parquet metadata nests too deeply");
    switch (type) {
      case CT_TRUE:
      case CT_FALSE: return;
      case CT_BYTE: byte(); return;
      case CT_I16:
      case CT_I32:
      case CT_I64: varint(); return;
      case CT_DOUBLE:
        for (int i = 0; i < 8; ++i) byte();
        return;
      case CT_BINARY: binary(); return;
      case CT_LIST:
      case CT_SET: {
        int elem = 0;
        const int64_t n = list(&elem);
        for (int64_t i = 0; i < n; ++i) skip_element(elem, depth + 1);
        return;
      }
      case CT_MAP: {
        const int64_t n = static_cast<int64_t>(varint());
        if (n == 0) return;
        const uint8_t kv = byte();
        for (int64_t i = 0; i < n; ++i) {
          skip_element(kv >> 4, depth + 1);
          skip_element(kv & 0x0f, depth + 1);
        }
        return;
      }
      case CT_STRUCT: {
        int16_t last = 0;
        int id, t;
        while (field(&last, &id, &t)) skip(t, depth + 1);
        return;
      }
      default: fail(GFPDB_EINVAL, "Parquet metadata: unknown Thrift type " + std::to_string(type));
    }
  }

 private:
  const uint8_t* p_;
  int64_t n_;
  int64_t pos_ = 0;
};

struct SchemaEl {
  std::string name;
  int32_t type = -1, repetition = 0, num_children = 0, converted = -1;
  bool logical_date = false, logical_string = false;
};

SchemaEl read_schema_element(Reader& r) {
  SchemaEl e;
  int16_t last = 0;
  int id, t;
  while (r.field(&last, &id, &t)) {
    switch (id) {
      case 1: e.type = static_cast<int32_t>(r.zigzag()); break;
      case 3: e.repetition = static_cast<int32_t>(r.zigzag()); break;
      case 4: e.name = r.binary(); break;
      case 5: e.num_children = static_cast<int32_t>(r.zigzag()); break;
      case 6: e.converted = static_cast<int32_t>(r.zigzag()); break;
      case 10: {  // LogicalType: a union, one field set (1 STRING, 6 DATE)
        int16_t l2 = 0;
        int id2, t2;
        while (r.field(&l2, &id2, &t2)) {
          if (id2 == 1) e.logical_string = true;
          if (id2 == 6) e.logical_date = true;
          r.skip(t2);
        }
        break;
      }
      default: r.skip(t);
    }
  }
  return e;
}

struct ChunkMeta {
  int32_t codec = 0;
  int64_t num_values = 0, total_compressed = 0, data_page_offset = 0, dict_page_offset = -1, null_count = -1;
};

int64_t read_statistics_nulls(Reader& r) {
  int64_t nulls = -1;
  int16_t last = 0;
  int id, t;
  while (r.field(&last, &id, &t)) {
    if (id == 3 && t == CT_I64) nulls = r.zigzag();
    else r.skip(t);
  }
  return nulls;
}

ChunkMeta read_column_meta(Reader& r) {
  ChunkMeta m;
  int16_t last = 0;
  int id, t;
  while (r.field(&last, &id, &t)) {
    switch (id) {
      case 4: m.codec = static_cast<int32_t>(r.zigzag()); break;
      case 5: m.num_values = r.zigzag(); break;
      case 7: m.total_compressed = r.zigzag(); break;
      case 9: m.data_page_offset = r.zigzag(); break;
      case 11: m.dict_page_offset = r.zigzag(); break;
      case 12: m.null_count = read_statistics_nulls(r); break;
      default: r.skip(t);
    }
  }
  return m;
}

struct RowGroupMeta {
  std::vector<ChunkMeta> chunks;
  int64_t num_rows = 0;
};

RowGroupMeta read_row_group(Reader& r) {
  RowGroupMeta g;
  int16_t last = 0;
  int id, t;
  while (r.field(&last, &id, &t)) {
    if (id == 1 && t == CT_LIST) {
      int elem;
      const int64_t n = r.list(&elem);
      for (int64_t i = 0; i < n; ++i) {
        ChunkMeta cm;
        int16_t l2 = 0;
        int id2, t2;
        bool has_meta = false;
        while (r.field(&l2, &id2, &t2)) {
          if (id2 == 1) fail(GFPDB_EUNSUPPORTED, "Parquet column chunks in other files");
          if (id2 == 3 && t2 == CT_STRUCT) {
            cm = read_column_meta(r);
            has_meta = true;
          } else {
            r.skip(t2);
          }
        }
        if (!has_meta) fail(GFPDB_EINVAL, "Parquet column chunk without metadata");
        g.chunks.push_back(cm);
      }
    } else if (id == 3) {
      g.num_rows = r.zigzag();
    } else {
      r.skip(t);
    }
  }
  return g;
}

struct PageHeaderMeta {
  int32_t type = 0, uncompressed = 0, compressed = 0;
  int32_t num_values = 0, encoding = 0, num_nulls = 0, def_len = 0, rep_len = 0;
  bool v2_compressed = true;
  int64_t stats_nulls = -1;
};

PageHeaderMeta read_page_header(Reader& r) {
  PageHeaderMeta h;
  int16_t last = 0;
  int id, t;
  while (r.field(&last, &id, &t)) {
    switch (id) {
      case 1: h.type = static_cast<int32_t>(r.zigzag()); break;
      case 2: h.uncompressed = static_cast<int32_t>(r.zigzag()); break;
      case 3: h.compressed = static_cast<int32_t>(r.zigzag()); break;
      case 5:    // DataPageHeader
      case 7:    // DictionaryPageHeader
      case 8: {  // DataPageHeaderV2
        int16_t l2 = 0;
        int id2, t2;
        while (r.field(&l2, &id2, &t2)) {
          if (id2 == 1) {
            h.num_values = static_cast<int32_t>(r.zigzag());
          } else if (id == 8 && id2 == 2) {
            h.num_nulls = static_cast<int32_t>(r.zigzag());
          } else if ((id == 5 && id2 == 2) || (id == 7 && id2 == 2) || (id == 8 && id2 == 4)) {
            h.encoding = static_cast<int32_t>(r.zigzag());
          } else if (id == 8 && id2 == 5) {
            h.def_len = static_cast<int32_t>(r.zigzag());
          } else if (id == 8 && id2 == 6) {
            h.rep_len = static_cast<int32_t>(r.zigzag());
          } else if (id == 8 && id2 == 7) {
            h.v2_compressed = r.boolean(t2);
          } else if (id == 5 && id2 == 5 && t2 == CT_STRUCT) {
            h.stats_nulls = read_statistics_nulls(r);
          } else {
            r.skip(t2);
          }
        }
        break;
      }
      default: r.skip(t);
    }
  }
  return h;
}

DType dtype_of(const SchemaEl& e) {
  switch (e.type) {
    case PT_INT32: return (e.converted == 6 || e.logical_date) ? DType::Date32 : DType::Int32;
    case PT_INT64: return DType::Int64;
    case PT_DOUBLE: return DType::Float64;
    case PT_BYTE_ARRAY: return DType::Utf8;
    default:
      fail(GFPDB_EUNSUPPORTED, "Parquet column '" + e.name + "' of physical type " + std::to_string(e.type) +
                                   " (BOOLEAN, INT96, FLOAT and FIXED_LEN_BYTE_ARRAY are not read)");
  }
}

}  // namespace

Layout read_layout(const uint8_t* file, int64_t size, const std::vector<std::string>& names, int64_t start_pos,
                   int64_t end_pos) {
  if (size < 12 || std::memcmp(file, "PAR1", 4) != 0 || std::memcmp(file + size - 4, "PAR1", 4) != 0)
    fail(GFPDB_EINVAL, "not a Parquet file (no PAR1 magic)");
  uint32_t footer_len = 0;
  std::memcpy(&footer_len, file + size - 8, 4);  // little-endian on every host this builds for
  if (footer_len > static_cast<uint64_t>(size - 12)) fail(GFPDB_EINVAL, "Parquet footer length out of range");
  Reader r(file + size - 8 - footer_len, footer_len);

  std::vector<SchemaEl> schema;
  std::vector<RowGroupMeta> groups;
  int16_t last = 0;
  int id, t;
  while (r.field(&last, &id, &t)) {
    if (id == 2 && t == CT_LIST) {
      int elem;
      const int64_t n = r.list(&elem);
      for (int64_t i = 0; i < n; ++i) schema.push_back(read_schema_element(r));
    } else if (id == 4 && t == CT_LIST) {
      int elem;
      const int64_t n = r.list(&elem);
      for (int64_t i = 0; i < n; ++i) groups.push_back(read_row_group(r));
    } else {
      r.skip(t);
    }
  }
  if (schema.empty()) fail(GFPDB_EINVAL, "Parquet schema is empty");
  // a flat schema: the root, then one leaf per column
  std::vector<SchemaEl> leaves(schema.begin() + 1, schema.end());
  for (auto& e : leaves) {
    // names travel into Arrow schemas, whose names are UTF-8
    if (!valid_utf8(e.name)) fail(GFPDB_EINVAL, "Parquet column name is not UTF-8");
    if (e.num_children > 0) fail(GFPDB_EUNSUPPORTED, "nested Parquet columns ('" + e.name + "')");
    if (e.repetition == 2) fail(GFPDB_EUNSUPPORTED, "repeated Parquet column '" + e.name + "'");
  }

  Layout L;
  std::vector<int> picked;
  if (names.empty()) {
    for (size_t i = 0; i < leaves.size(); ++i) picked.push_back(static_cast<int>(i));
  } else {
    for (auto& n : names) {
      auto it = std::find_if(leaves.begin(), leaves.end(), [&](const SchemaEl& e) { return e.name == n; });
      if (it == leaves.end()) fail(GFPDB_EINVAL, "Read Parquet Error: column " + n + " not found");
      picked.push_back(static_cast<int>(it - leaves.begin()));
    }
  }
  for (int ci : picked) {
    const SchemaEl& e = leaves[ci];
    ColumnInfo c;
    c.name = e.name;
    c.physical = e.type;
    c.repetition = e.repetition;
    c.converted = e.converted;
    c.logical_date = e.logical_date;
    c.logical_string = e.logical_string;
    c.dtype = dtype_of(e);
    L.columns.push_back(c);
  }

  std::vector<int64_t> rows_so_far(picked.size(), 0);
  for (const auto& g : groups) {
    if (g.chunks.size() != leaves.size()) fail(GFPDB_EINVAL, "Parquet row group column count disagrees with the schema");
    const ChunkMeta& first = g.chunks[0];
    const int64_t first_off = first.dict_page_offset > 0 && first.dict_page_offset < first.data_page_offset
                                  ? first.dict_page_offset
                                  : first.data_page_offset;
    if (start_pos <= end_pos && (first_off < start_pos || first_off > end_pos)) continue;
    L.row_groups.push_back(RowGroupInfo{first_off, g.num_rows});
    L.num_rows += g.num_rows;
    for (size_t k = 0; k < picked.size(); ++k) {
      const ChunkMeta& m = g.chunks[picked[k]];
      const ColumnInfo& c = L.columns[k];
      if (m.codec != CODEC_UNCOMPRESSED && m.codec != CODEC_SNAPPY)
        fail(GFPDB_EUNSUPPORTED, "Parquet codec " + std::to_string(m.codec) + " of column '" + c.name +
                                     "' (uncompressed and snappy are read)");
      if (m.null_count > 0)
        fail(GFPDB_EUNSUPPORTED, "Parquet column '" + c.name + "' has nulls; nullable inputs are not supported");
      int64_t pos = m.dict_page_offset > 0 && m.dict_page_offset < m.data_page_offset ? m.dict_page_offset
                                                                                       : m.data_page_offset;
      const int64_t end = pos + m.total_compressed;
      if (pos < 4 || end > size - 8 - static_cast<int64_t>(footer_len))
        fail(GFPDB_EINVAL, "Parquet column chunk of '" + c.name + "' lies outside the file");
      int32_t dict = -1;
      int64_t values = 0;
      const int32_t chunk_id = static_cast<int32_t>(L.chunks.size());
      L.chunks.push_back(ChunkRange{pos, end});
      while (pos < end && values < m.num_values) {
        Reader hr(file + pos, end - pos);
        const PageHeaderMeta h = read_page_header(hr);
        PageInfo pg;
        pg.column = static_cast<int32_t>(k);
        pg.chunk = chunk_id;
        pg.type = h.type;
        pg.codec = m.codec;
        pg.data_offset = pos + hr.pos();
        pg.compressed = h.compressed;
        pg.uncompressed = h.uncompressed;
        pg.num_values = h.num_values;
        pg.encoding = h.encoding;
        if (h.compressed < 0 || h.uncompressed < 0 || pg.data_offset + h.compressed > end)
          fail(GFPDB_EINVAL, "Parquet page of '" + c.name + "' runs past its column chunk");
        pos = pg.data_offset + h.compressed;
        if (h.type == PAGE_INDEX) continue;
        if (h.type == PAGE_DICTIONARY) {
          if (h.encoding != ENC_PLAIN && h.encoding != ENC_PLAIN_DICTIONARY)
            fail(GFPDB_EUNSUPPORTED, "Parquet dictionary encoding " + std::to_string(h.encoding));
          dict = static_cast<int32_t>(L.pages.size());
          L.pages.push_back(pg);
          continue;
        }
        if (h.type != PAGE_DATA && h.type != PAGE_DATA_V2)
          fail(GFPDB_EUNSUPPORTED, "Parquet page type " + std::to_string(h.type));
        if (h.encoding != ENC_PLAIN && h.encoding != ENC_PLAIN_DICTIONARY && h.encoding != ENC_RLE_DICTIONARY)
          fail(GFPDB_EUNSUPPORTED, "Parquet encoding " + std::to_string(h.encoding) + " of column '" + c.name +
                                       "' (plain and dictionary are read)");
        if (h.encoding != ENC_PLAIN && dict < 0)
          fail(GFPDB_EINVAL, "Parquet dictionary-encoded page without a dictionary page");
        if ((h.type == PAGE_DATA_V2 && h.num_nulls > 0) || h.stats_nulls > 0)
          fail(GFPDB_EUNSUPPORTED, "Parquet column '" + c.name + "' has nulls; nullable inputs are not supported");
        if (h.type == PAGE_DATA_V2) {
          if (h.rep_len != 0) fail(GFPDB_EUNSUPPORTED, "repeated Parquet column '" + c.name + "'");
          pg.v2_levels = h.def_len;
          pg.v2_compressed = h.v2_compressed;
          if (h.def_len > h.compressed) fail(GFPDB_EINVAL, "Parquet page levels exceed the page");
        } else {
          pg.v1_def_levels = c.repetition == 1;
        }
        pg.dict_page = h.encoding == ENC_PLAIN ? -1 : dict;
        pg.first_row = rows_so_far[k];
        rows_so_far[k] += h.num_values;
        values += h.num_values;
        L.pages.push_back(pg);
      }
      if (values != m.num_values) fail(GFPDB_EINVAL, "Parquet column chunk of '" + c.name + "' is short of values");
    }
  }
  for (size_t k = 0; k < picked.size(); ++k)
    if (rows_so_far[k] != L.num_rows) fail(GFPDB_EINVAL, "Parquet column '" + L.columns[k].name + "' row count");
  return L;
}

}  // namespace gfpdb::parquet
