// Device-resident TupleSet: the GPU form of fpdb::tuple::TupleSet
// (fpdb-tuple/include/fpdb/tuple/TupleSet.h:31-207).
//
// The reference wraps an arrow::Table of chunked columns that operators share
// by shared_ptr and never mutate after sending (concatenate instead of append,
// fpdb-executor/src/physical/bloomfilter/BloomFilterCreateAbstractKernel.cpp:22-38).
// Here each column is one contiguous device buffer (Arrow layout: values for
// fixed-width types, int32 offsets + bytes for utf8); columns are immutable and
// shared between TupleSets by shared_ptr, so projection is free and a
// TupleSet sent to several consumers is never copied.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "runtime.h"

namespace gfpdb {

enum class DType : int8_t { Int32 = 0, Int64 = 1, Date32 = 2, Float64 = 3, Utf8 = 4 };

const char* dtype_name(DType t);
int dtype_width(DType t);  // bytes per value; 0 for utf8
DType dtype_from_format(const char* format);
const char* dtype_format(DType t);
DType dtype_from_name(const std::string& name);  // "int32", "int64", "date32", "float64", "utf8"

struct Column {
  DType type = DType::Int32;
  int64_t length = 0;
  BufferPtr data_buf;      // keeps the value (or utf8 byte) memory alive
  BufferPtr offsets_buf;   // utf8 only
  const void* data = nullptr;        // first value of this column
  const int32_t* offsets = nullptr;  // utf8: length + 1 offsets into `data`
  // Validity (outer-join outputs only): bit i of the LSB-first words is 1
  // when row i holds a value (Arrow's bitmap order); none means no nulls.
  BufferPtr valid_buf;
  const uint32_t* valid = nullptr;

  int64_t value_bytes() const;  // bytes of values (utf8: bytes spanned by offsets)
};
using ColumnPtr = std::shared_ptr<const Column>;

struct Field {
  std::string name;
  DType type;
};

class TupleSet;
using TupleSetPtr = std::shared_ptr<const TupleSet>;

class TupleSet {
 public:
  TupleSet(std::vector<Field> fields, std::vector<ColumnPtr> columns, int64_t num_rows);

  static TupleSetPtr make(std::vector<Field> fields, std::vector<ColumnPtr> columns, int64_t num_rows);
  static TupleSetPtr make_empty(const std::vector<Field>& fields, cudaStream_t s);

  // A TupleSet whose true row count is only known on the device (written
  // there by the kernel that produced it): `capacity` rows of every column
  // are allocated and *rows_dev holds the count. Operators chained on the
  // same stream consume it without a host round trip; resolve() reads the
  // count when the host needs it.
  static TupleSetPtr make_deferred(std::vector<Field> fields, std::vector<ColumnPtr> columns, int64_t capacity,
                                   BufferPtr rows_owner, const int64_t* rows_dev);
  bool exact() const { return rows_dev_ == nullptr; }
  const int64_t* rows_dev() const { return rows_dev_; }
  const BufferPtr& rows_owner() const { return rows_owner_; }
  // Same columns with the exact row count (synchronizes `s` when deferred).
  TupleSetPtr resolve(cudaStream_t s) const;

  // Exact row count, or the capacity (upper bound) of a deferred TupleSet.
  int64_t num_rows() const { return num_rows_; }
  int num_columns() const { return static_cast<int>(columns_.size()); }
  const std::vector<Field>& fields() const { return fields_; }
  const Field& field(int i) const { return fields_.at(i); }
  const ColumnPtr& column(int i) const { return columns_.at(i); }
  int column_index(const std::string& name) const;  // -1 when absent
  int require_column(const std::string& name) const;  // throws GFPDB_EINVAL
  ColumnPtr column(const std::string& name) const { return columns_[require_column(name)]; }

  // Keep the named columns that exist, in the given order
  // (TupleSet::projectExist, fpdb-tuple/src/TupleSet.cpp).
  TupleSetPtr project_exist(const std::vector<std::string>& names) const;
  TupleSetPtr project(const std::vector<std::string>& names) const;  // all must exist

  int64_t bytes() const;

  // Row-wise concatenation into fresh device buffers
  // (TupleSet::concatenate, fpdb-tuple/src/TupleSet.cpp).
  static TupleSetPtr concatenate(const std::vector<TupleSetPtr>& sets, cudaStream_t s);

 private:
  std::vector<Field> fields_;
  std::vector<ColumnPtr> columns_;
  int64_t num_rows_;
  BufferPtr rows_owner_;
  const int64_t* rows_dev_ = nullptr;
};

// `ts` itself when exact, else its resolved copy (synchronizes `s`).
inline TupleSetPtr resolved(const TupleSetPtr& ts, cudaStream_t s) { return ts->exact() ? ts : ts->resolve(s); }

// Column factories.
ColumnPtr make_fixed_column(DType t, int64_t length, BufferPtr buf, const void* data = nullptr);
ColumnPtr make_utf8_column(int64_t length, BufferPtr offsets, BufferPtr bytes);
// The same column with a validity bitmap ((length + 31) / 32 words).
ColumnPtr with_validity(const ColumnPtr& c, BufferPtr bits);
// Whether any column may hold nulls (has a validity bitmap).
bool has_nulls(const TupleSet& ts);
std::string first_nullable_column(const TupleSet& ts);  // "" when none

// ---- Arrow C Data / Device Data Interface ----

// Import a struct-typed (ArrowSchema "+s", ArrowDeviceArray) pair. Device
// arrays are borrowed (the caller keeps them alive for the duration of the
// call) unless copy_device is set; host arrays are copied to the device on
// stream `s`.
// Device address of page-locked host memory (nullptr for pageable memory).
const void* device_view_of_host(const void* p);

// `wanted` (when given) limits the import to those columns (schema order
// kept); the columns named in `in_place` of a page-locked host table are not
// copied: kernels read them over the chip-to-chip link (a column of pageable
// memory is copied all the same).
TupleSetPtr import_tupleset(const ArrowSchema* schema, const ArrowDeviceArray* array, cudaStream_t s,
                            bool copy_device = false, const std::vector<std::string>* wanted = nullptr,
                            const std::vector<std::string>* in_place = nullptr);
std::vector<Field> import_schema(const ArrowSchema* schema);

// Export a TupleSet. With to_host, values are copied to host memory (stream
// synchronized) and the array's device_type is ARROW_DEVICE_CPU.
void export_tupleset(const TupleSetPtr& ts, ArrowSchema* schema_out, ArrowDeviceArray* array_out,
                     bool to_host, cudaStream_t s);

// Export columns that already sit in host memory (copied into fresh host
// allocations). Per column: {values} for fixed-width types, {offsets, bytes}
// for utf8 (offsets are rebased to start at 0).
void export_host_columns(const std::vector<Field>& fields, int64_t n,
                         const std::vector<std::vector<const void*>>& bufs, ArrowSchema* schema_out,
                         ArrowDeviceArray* array_out);

}  // namespace gfpdb
