// Parquet file metadata on the host: the footer (FileMetaData) and each
// column chunk's page headers, decoded from the Thrift compact protocol, as
// the list of pages the device decoder works through.
//
// This replaces the metadata half of Arrow's parquet::arrow::FileReader that
// ParquetReader::readImpl / readRangeImpl drive
// (fpdb-tuple/src/parquet/ParquetReader.cpp:12-120); the layout follows the
// public Apache Parquet format specification (parquet.thrift: FileMetaData,
// SchemaElement, RowGroup, ColumnChunk, ColumnMetaData, PageHeader and its
// data / dictionary / data-v2 headers).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "tupleset.h"

namespace gfpdb::parquet {

// parquet.thrift enums (the values are the format's)
enum PhysicalType : int32_t { PT_BOOLEAN = 0, PT_INT32 = 1, PT_INT64 = 2, PT_INT96 = 3, PT_FLOAT = 4, PT_DOUBLE = 5,
                              PT_BYTE_ARRAY = 6, PT_FIXED_LEN_BYTE_ARRAY = 7 };
enum Codec : int32_t { CODEC_UNCOMPRESSED = 0, CODEC_SNAPPY = 1 };
enum Encoding : int32_t { ENC_PLAIN = 0, ENC_PLAIN_DICTIONARY = 2, ENC_RLE = 3, ENC_RLE_DICTIONARY = 8 };
enum PageType : int32_t { PAGE_DATA = 0, PAGE_INDEX = 1, PAGE_DICTIONARY = 2, PAGE_DATA_V2 = 3 };

struct ColumnInfo {
  std::string name;
  int32_t physical = PT_INT32;
  int32_t repetition = 0;  // 0 REQUIRED, 1 OPTIONAL, 2 REPEATED
  int32_t converted = -1;  // ConvertedType (UTF8 = 0, DATE = 6), -1 when absent
  bool logical_date = false;
  bool logical_string = false;
  DType dtype = DType::Int32;  // the TupleSet type it decodes to
};

// One page of one selected column, in row order.
struct PageInfo {
  int32_t column = 0;        // index into the selected columns
  int32_t type = PAGE_DATA;  // PageType
  int32_t encoding = ENC_PLAIN;
  int32_t codec = CODEC_UNCOMPRESSED;
  int64_t data_offset = 0;   // file offset of the page body (after its header)
  int32_t compressed = 0;    // bytes of the body in the file
  int32_t uncompressed = 0;  // bytes after decompression
  int32_t num_values = 0;
  int32_t v2_levels = 0;     // data page v2: level bytes before the values (never compressed)
  bool v2_compressed = true;
  bool v1_def_levels = false;  // data page v1 of an optional column: a 4-byte length then RLE levels
  int64_t first_row = 0;     // row of the page's first value within the column
  int32_t dict_page = -1;    // data pages: index of their chunk's dictionary page in the page list
  int32_t chunk = 0;         // index into Layout::chunks
};

// The bytes of one column chunk in the file (its pages and their headers).
struct ChunkRange {
  int64_t begin = 0, end = 0;
};

// A selected row group: the file offset of its first column chunk (the
// position readRange selects it by) and its rows.
struct RowGroupInfo {
  int64_t offset = 0;
  int64_t rows = 0;
};

struct Layout {
  std::vector<ColumnInfo> columns;  // the selected columns, in the requested order
  std::vector<PageInfo> pages;
  std::vector<ChunkRange> chunks;
  std::vector<RowGroupInfo> row_groups;
  int64_t num_rows = 0;             // rows of the selected row groups
};

// The footer and page headers of a whole file held in host memory. Columns
// are selected by name (all when `names` is empty); with start_pos <= end_pos
// only the row groups whose first column chunk starts within [start_pos,
// end_pos] are read (ParquetReader::readRangeImpl,
// fpdb-tuple/src/parquet/ParquetReader.cpp:44-77). Unsupported features
// (nested or repeated columns, nulls, codecs other than none and snappy,
// encodings other than plain and dictionary, BOOLEAN / INT96 / FLOAT /
// FIXED_LEN_BYTE_ARRAY columns) raise GFPDB_EUNSUPPORTED.
Layout read_layout(const uint8_t* file, int64_t size, const std::vector<std::string>& names, int64_t start_pos = 0,
                   int64_t end_pos = -1);

}  // namespace gfpdb::parquet
