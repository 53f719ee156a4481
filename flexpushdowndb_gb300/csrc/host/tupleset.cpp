#include "tupleset.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "../kernels/launch.h"

namespace gfpdb {

const char* dtype_name(DType t) {
  switch (t) {
    case DType::Int32: return "int32";
    case DType::Int64: return "int64";
    case DType::Date32: return "date32";
    case DType::Float64: return "float64";
    case DType::Utf8: return "utf8";
  }
  return "?";
}

int dtype_width(DType t) {
  switch (t) {
    case DType::Int32: return 4;
    case DType::Int64: return 8;
    case DType::Date32: return 4;
    case DType::Float64: return 8;
    case DType::Utf8: return 0;
  }
  return 0;
}

DType dtype_from_format(const char* f) {
  if (f == nullptr) fail(GFPDB_EINVAL, "ArrowSchema child without a format");
  if (std::strcmp(f, "i") == 0) return DType::Int32;
  if (std::strcmp(f, "l") == 0) return DType::Int64;
  if (std::strcmp(f, "tdD") == 0) return DType::Date32;
  if (std::strcmp(f, "g") == 0) return DType::Float64;
  if (std::strcmp(f, "u") == 0) return DType::Utf8;
  fail(GFPDB_EUNSUPPORTED, std::string("unsupported Arrow format '") + f + "'");
}

const char* dtype_format(DType t) {
  switch (t) {
    case DType::Int32: return "i";
    case DType::Int64: return "l";
    case DType::Date32: return "tdD";
    case DType::Float64: return "g";
    case DType::Utf8: return "u";
  }
  return "";
}

DType dtype_from_name(const std::string& n) {
  if (n == "int32" || n == "Int32") return DType::Int32;
  if (n == "int64" || n == "Int64") return DType::Int64;
  if (n == "date32" || n == "Date32") return DType::Date32;
  if (n == "float64" || n == "double" || n == "Double") return DType::Float64;
  if (n == "utf8" || n == "string") return DType::Utf8;
  fail(GFPDB_EUNSUPPORTED, "unsupported data type '" + n + "'");
}

int64_t Column::value_bytes() const {
  if (type == DType::Utf8) return 0;  // needs the offsets on the host; not used for sizing
  return length * dtype_width(type);
}

ColumnPtr make_fixed_column(DType t, int64_t length, BufferPtr buf, const void* data) {
  auto c = std::make_shared<Column>();
  c->type = t;
  c->length = length;
  c->data = data != nullptr ? data : buf->data();
  c->data_buf = std::move(buf);
  return c;
}

ColumnPtr with_validity(const ColumnPtr& c, BufferPtr bits) {
  auto v = std::make_shared<Column>(*c);
  v->valid = bits ? bits->as<uint32_t>() : nullptr;
  v->valid_buf = std::move(bits);
  return v;
}

bool has_nulls(const TupleSet& ts) { return !first_nullable_column(ts).empty(); }

std::string first_nullable_column(const TupleSet& ts) {
  for (int i = 0; i < ts.num_columns(); ++i)
    if (ts.column(i)->valid != nullptr) return ts.field(i).name;
  return "";
}

ColumnPtr make_utf8_column(int64_t length, BufferPtr offsets, BufferPtr bytes) {
  auto c = std::make_shared<Column>();
  c->type = DType::Utf8;
  c->length = length;
  c->offsets = offsets->as<int32_t>();
  c->data = bytes->data();
  c->offsets_buf = std::move(offsets);
  c->data_buf = std::move(bytes);
  return c;
}

TupleSet::TupleSet(std::vector<Field> fields, std::vector<ColumnPtr> columns, int64_t num_rows)
    : fields_(std::move(fields)), columns_(std::move(columns)), num_rows_(num_rows) {
  if (fields_.size() != columns_.size()) fail(GFPDB_EINVAL, "TupleSet: field/column count mismatch");
  for (size_t i = 0; i < columns_.size(); ++i) {
    if (columns_[i]->length != num_rows_) fail(GFPDB_EINVAL, "TupleSet: ragged columns");
    if (columns_[i]->type != fields_[i].type) fail(GFPDB_EINVAL, "TupleSet: column type mismatch");
  }
}

TupleSetPtr TupleSet::make(std::vector<Field> fields, std::vector<ColumnPtr> columns, int64_t num_rows) {
  return std::make_shared<const TupleSet>(std::move(fields), std::move(columns), num_rows);
}

TupleSetPtr TupleSet::make_deferred(std::vector<Field> fields, std::vector<ColumnPtr> columns, int64_t capacity,
                                    BufferPtr rows_owner, const int64_t* rows_dev) {
  auto ts = std::make_shared<TupleSet>(std::move(fields), std::move(columns), capacity);
  ts->rows_owner_ = std::move(rows_owner);
  ts->rows_dev_ = rows_dev;
  return ts;
}

TupleSetPtr TupleSet::resolve(cudaStream_t s) const {
  if (exact()) return make(fields_, columns_, num_rows_);
  int64_t n = 0;
  GF_CUDA(cudaMemcpyAsync(&n, rows_dev_, sizeof(n), cudaMemcpyDeviceToHost, s));
  sync(s);
  if (n < 0 || n > num_rows_) fail(GFPDB_EDEVICE, "deferred row count out of range");
  std::vector<ColumnPtr> cols;
  for (auto& c : columns_) {
    auto r = std::make_shared<Column>(*c);
    r->length = n;
    cols.push_back(r);
  }
  return make(fields_, std::move(cols), n);
}

TupleSetPtr TupleSet::make_empty(const std::vector<Field>& fields, cudaStream_t s) {
  std::vector<ColumnPtr> cols;
  for (auto& f : fields) {
    if (f.type == DType::Utf8) {
      auto off = make_buffer(4, s);
      GF_CUDA(cudaMemsetAsync(off->data(), 0, 4, s));
      cols.push_back(make_utf8_column(0, off, make_buffer(0, s)));
    } else {
      cols.push_back(make_fixed_column(f.type, 0, make_buffer(0, s)));
    }
  }
  return make(fields, std::move(cols), 0);
}

int TupleSet::column_index(const std::string& name) const {
  for (size_t i = 0; i < fields_.size(); ++i)
    if (fields_[i].name == name) return static_cast<int>(i);
  return -1;
}

int TupleSet::require_column(const std::string& name) const {
  int i = column_index(name);
  if (i < 0) fail(GFPDB_EINVAL, "column '" + name + "' not found in TupleSet");
  return i;
}

TupleSetPtr TupleSet::project_exist(const std::vector<std::string>& names) const {
  std::vector<Field> f;
  std::vector<ColumnPtr> c;
  for (auto& n : names) {
    int i = column_index(n);
    if (i >= 0) {
      f.push_back(fields_[i]);
      c.push_back(columns_[i]);
    }
  }
  if (exact()) return make(std::move(f), std::move(c), num_rows_);
  return make_deferred(std::move(f), std::move(c), num_rows_, rows_owner_, rows_dev_);
}

TupleSetPtr TupleSet::project(const std::vector<std::string>& names) const {
  std::vector<Field> f;
  std::vector<ColumnPtr> c;
  for (auto& n : names) {
    int i = require_column(n);
    f.push_back(fields_[i]);
    c.push_back(columns_[i]);
  }
  if (exact()) return make(std::move(f), std::move(c), num_rows_);
  return make_deferred(std::move(f), std::move(c), num_rows_, rows_owner_, rows_dev_);
}

int64_t TupleSet::bytes() const {
  int64_t b = 0;
  for (auto& c : columns_) b += c->type == DType::Utf8 ? (c->length + 1) * 4 : c->value_bytes();
  return b;
}

TupleSetPtr TupleSet::concatenate(const std::vector<TupleSetPtr>& sets, cudaStream_t s) {
  if (sets.empty()) fail(GFPDB_EINVAL, "concatenate: no TupleSets");
  if (sets.size() == 1) return sets[0];
  for (auto& t : sets)
    if (!t->exact()) {
      std::vector<TupleSetPtr> exact_sets;
      for (auto& u : sets) exact_sets.push_back(resolved(u, s));
      return concatenate(exact_sets, s);
    }
  const auto& fields = sets[0]->fields();
  int64_t total = 0;
  for (auto& t : sets) {
    if (t->num_columns() != static_cast<int>(fields.size())) fail(GFPDB_EINVAL, "concatenate: schema mismatch");
    for (int i = 0; i < t->num_columns(); ++i)
      if (t->field(i).type != fields[i].type || t->field(i).name != fields[i].name)
        fail(GFPDB_EINVAL, "concatenate: schema mismatch on column '" + fields[i].name + "'");
    total += t->num_rows();
  }
  std::vector<ColumnPtr> cols;
  for (size_t ci = 0; ci < fields.size(); ++ci) {
    DType t = fields[ci].type;
    if (t != DType::Utf8) {
      int w = dtype_width(t);
      auto buf = make_buffer(total * w, s);
      int64_t at = 0;
      for (auto& ts : sets) {
        const auto& c = ts->column(static_cast<int>(ci));
        if (c->length > 0)
          GF_CUDA(cudaMemcpyAsync(buf->as<char>() + at * w, c->data, c->length * w, cudaMemcpyDeviceToDevice, s));
        at += c->length;
      }
      cols.push_back(make_fixed_column(t, total, buf));
    } else {
      std::vector<const Column*> parts;
      for (auto& ts : sets) parts.push_back(ts->column(static_cast<int>(ci)).get());
      cols.push_back(concat_utf8(parts, s));
    }
    bool nullable = false;
    for (auto& ts : sets) nullable |= ts->column(static_cast<int>(ci))->valid != nullptr;
    if (nullable) {
      std::vector<std::pair<const uint32_t*, int64_t>> parts;
      for (auto& ts : sets) parts.emplace_back(ts->column(static_cast<int>(ci))->valid, ts->num_rows());
      cols.back() = with_validity(cols.back(), validity_concat(parts, total, s));
    }
  }
  return make(fields, std::move(cols), total);
}

// ---------------------------------------------------------------- import

std::vector<Field> import_schema(const ArrowSchema* schema) {
  if (schema == nullptr || schema->release == nullptr) fail(GFPDB_EINVAL, "null or released ArrowSchema");
  if (schema->format == nullptr || std::strcmp(schema->format, "+s") != 0)
    fail(GFPDB_EINVAL, "a TupleSet schema must be a struct (format \"+s\")");
  if (schema->n_children < 0 || (schema->n_children > 0 && schema->children == nullptr))
    fail(GFPDB_EINVAL, "ArrowSchema with a negative child count or without its children");
  std::vector<Field> fields;
  for (int64_t i = 0; i < schema->n_children; ++i) {
    const ArrowSchema* c = schema->children[i];
    if (c == nullptr || c->release == nullptr)
      fail(GFPDB_EINVAL, "ArrowSchema child " + std::to_string(i) + " is missing or released");
    fields.push_back(Field{c->name != nullptr ? c->name : "", dtype_from_format(c->format)});
  }
  return fields;
}

// Device address of page-locked host memory (nullptr for pageable memory).
const void* device_view_of_host(const void* p) {
  cudaPointerAttributes attr{};
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  if (attr.type != cudaMemoryTypeHost) return nullptr;
  return attr.devicePointer != nullptr ? attr.devicePointer : p;
}

TupleSetPtr import_tupleset(const ArrowSchema* schema, const ArrowDeviceArray* darr, cudaStream_t s,
                            bool copy_device, const std::vector<std::string>* wanted,
                            const std::vector<std::string>* in_place) {
  auto all_fields = import_schema(schema);
  auto listed = [](const std::vector<std::string>* v, const std::string& n) {
    return v != nullptr && std::find(v->begin(), v->end(), n) != v->end();
  };
  if (darr == nullptr) fail(GFPDB_EINVAL, "null ArrowDeviceArray");
  const ArrowArray& arr = darr->array;
  if (arr.release == nullptr) fail(GFPDB_EINVAL, "released ArrowArray");
  bool host = darr->device_type == ARROW_DEVICE_CPU || darr->device_type == ARROW_DEVICE_CUDA_HOST;
  if (!host && darr->device_type != ARROW_DEVICE_CUDA)
    fail(GFPDB_EUNSUPPORTED, "unsupported ArrowDeviceArray device_type " + std::to_string(darr->device_type));
  if (arr.null_count > 0) fail(GFPDB_EUNSUPPORTED, "struct-level nulls are not supported");
  if (arr.n_children != static_cast<int64_t>(all_fields.size()))
    fail(GFPDB_EINVAL, "ArrowArray child count does not match the schema");
  const int64_t n = arr.length;
  const int64_t soff = arr.offset;
  if (n < 0 || soff < 0) fail(GFPDB_EINVAL, "ArrowArray with a negative length or offset");
  if (arr.n_children > 0 && arr.children == nullptr) fail(GFPDB_EINVAL, "ArrowArray without its children");
  std::vector<ColumnPtr> cols;
  std::vector<Field> fields;
  for (size_t i = 0; i < all_fields.size(); ++i) {
    if (wanted != nullptr && !listed(wanted, all_fields[i].name)) continue;
    fields.push_back(all_fields[i]);
    const ArrowArray* c = arr.children[i];
    if (c == nullptr || c->release == nullptr || c->buffers == nullptr || c->offset < 0)
      fail(GFPDB_EINVAL, "column '" + all_fields[i].name + "' is missing, released, without buffers or negatively offset");
    if (c->length < soff + n) fail(GFPDB_EINVAL, "column '" + all_fields[i].name + "' is shorter than the struct");
    if (c->null_count != 0 && c->buffers[0] != nullptr)
      fail(GFPDB_EUNSUPPORTED, "column '" + all_fields[i].name + "' has nulls; nullable inputs are not supported");
    const int64_t off = c->offset + soff;
    DType t = all_fields[i].type;
    if (t != DType::Utf8) {
      if (c->n_buffers != 2) fail(GFPDB_EINVAL, "fixed-width column needs 2 buffers");
      if (n > 0 && c->buffers[1] == nullptr) fail(GFPDB_EINVAL, "column '" + all_fields[i].name + "' has no values");
      int w = dtype_width(t);
      const char* src = static_cast<const char*>(c->buffers[1]) + off * w;
      const bool zero_copy = host && !copy_device && (host_copy_mode() == 2 || listed(in_place, all_fields[i].name));
      const void* zc = zero_copy ? device_view_of_host(src) : nullptr;
      if (zc != nullptr) {
        // Zero-copy: kernels read the page-locked host column over the
        // chip-to-chip link; only the sectors they touch cross it.
        auto buf = std::make_shared<DeviceBuffer>(const_cast<void*>(zc), n * w);
        cols.push_back(make_fixed_column(t, n, buf));
        copy_counters().in_place += n * w;
      } else if (host || copy_device) {
        auto buf = make_buffer(n * w, s);
        if (host) {
          copy_h2d(buf->data(), src, n * w, s);
        } else if (n > 0) {
          GF_CUDA(cudaMemcpyAsync(buf->data(), src, n * w, cudaMemcpyDeviceToDevice, s));
        }
        cols.push_back(make_fixed_column(t, n, buf));
      } else {
        auto buf = std::make_shared<DeviceBuffer>(const_cast<char*>(src), n * w);
        cols.push_back(make_fixed_column(t, n, buf));
      }
    } else {
      if (c->n_buffers != 3) fail(GFPDB_EINVAL, "utf8 column needs 3 buffers");
      const int32_t* offs = static_cast<const int32_t*>(c->buffers[1]) + off;
      const char* bytes = static_cast<const char*>(c->buffers[2]);
      if (host) {
        if (c->buffers[1] == nullptr) fail(GFPDB_EINVAL, "utf8 column '" + all_fields[i].name + "' has no offsets");
        // Offsets are rebased to start at 0 so the device copy holds only the
        // bytes this slice spans.
        int32_t first = offs[0], last = offs[n];
        if (first < 0 || last < first || (last > first && bytes == nullptr))
          fail(GFPDB_EINVAL, "utf8 column '" + all_fields[i].name + "' has offsets out of order or no bytes");
        std::vector<int32_t> rebased(n + 1);
        for (int64_t k = 0; k <= n; ++k) rebased[k] = offs[k] - first;
        auto ob = make_buffer((n + 1) * 4, s);
        auto bb = make_buffer(last - first, s);
        memcpy_h2d(ob->data(), rebased.data(), (n + 1) * 4, s);
        memcpy_h2d(bb->data(), bytes + first, last - first, s);
        // The rebased vector must outlive the async copy.
        sync(s);
        cols.push_back(make_utf8_column(n, ob, bb));
      } else if (copy_device) {
        Column tmp;
        tmp.type = DType::Utf8;
        tmp.length = n;
        tmp.offsets = offs;
        tmp.data = bytes;
        std::vector<const Column*> parts{&tmp};
        cols.push_back(concat_utf8(parts, s));
      } else {
        auto c2 = std::make_shared<Column>();
        c2->type = DType::Utf8;
        c2->length = n;
        c2->offsets = offs;
        c2->data = bytes;
        cols.push_back(c2);
      }
    }
  }
  return TupleSet::make(std::move(fields), std::move(cols), n);
}

// ---------------------------------------------------------------- export

namespace {

struct SchemaHolder {
  std::vector<std::string> names;
  std::vector<ArrowSchema> child_structs;
  std::vector<ArrowSchema*> child_ptrs;
};

void release_child_schema(ArrowSchema* s) { s->release = nullptr; }

void release_schema(ArrowSchema* s) {
  if (s == nullptr || s->release == nullptr) return;
  delete static_cast<SchemaHolder*>(s->private_data);
  s->release = nullptr;
}

struct ArrayHolder {
  TupleSetPtr ts;  // device memory stays alive while the array is alive
  std::vector<ArrowArray> child_structs;
  std::vector<ArrowArray*> child_ptrs;
  std::vector<std::vector<const void*>> child_buffers;
  std::vector<const void*> struct_buffers;
  std::vector<void*> host_allocs;  // host results
};

void release_child_array(ArrowArray* a) { a->release = nullptr; }

void release_array(ArrowArray* a) {
  if (a == nullptr || a->release == nullptr) return;
  auto* h = static_cast<ArrayHolder*>(a->private_data);
  for (void* p : h->host_allocs) std::free(p);
  delete h;
  a->release = nullptr;
}

}  // namespace

void export_tupleset(const TupleSetPtr& ts_in, ArrowSchema* so, ArrowDeviceArray* ao, bool to_host, cudaStream_t s) {
  const TupleSetPtr ts = resolved(ts_in, s);
  const int nc = ts->num_columns();
  // schema
  auto* sh = new SchemaHolder();
  sh->names.reserve(nc);
  sh->child_structs.resize(nc);
  sh->child_ptrs.resize(nc);
  for (int i = 0; i < nc; ++i) {
    sh->names.push_back(ts->field(i).name);
    ArrowSchema& c = sh->child_structs[i];
    std::memset(&c, 0, sizeof(c));
    c.format = dtype_format(ts->field(i).type);
    c.name = sh->names.back().c_str();
    c.flags = 0;
    c.release = release_child_schema;
    sh->child_ptrs[i] = &c;
  }
  std::memset(so, 0, sizeof(*so));
  so->format = "+s";
  so->name = "";
  so->n_children = nc;
  so->children = nc > 0 ? sh->child_ptrs.data() : nullptr;
  so->release = release_schema;
  so->private_data = sh;

  // array
  auto* ah = new ArrayHolder();
  ah->ts = ts;
  ah->child_structs.resize(nc);
  ah->child_ptrs.resize(nc);
  ah->child_buffers.resize(nc);
  const int64_t n = ts->num_rows();
  std::vector<std::pair<int, int64_t>> utf8_sizes;
  if (to_host) {
    // Copy the values to host memory; utf8 byte counts come from the last offset.
    std::vector<int32_t> last(nc, 0);
    for (int i = 0; i < nc; ++i) {
      const auto& c = ts->column(i);
      if (c->type == DType::Utf8 && n > 0) {
        int32_t ends[2] = {0, 0};
        memcpy_d2h(&ends[0], c->offsets, 4, s);
        memcpy_d2h(&ends[1], c->offsets + n, 4, s);
        sync(s);
        last[i] = ends[1] - ends[0];
        // rebase on the host after the copy
        int32_t* ho = static_cast<int32_t*>(std::malloc((n + 1) * 4));
        char* hb = static_cast<char*>(std::malloc(last[i] > 0 ? last[i] : 1));
        memcpy_d2h(ho, c->offsets, (n + 1) * 4, s);
        memcpy_d2h(hb, static_cast<const char*>(c->data) + ends[0], last[i], s);
        sync(s);
        for (int64_t k = 0; k <= n; ++k) ho[k] -= ends[0];
        ah->host_allocs.push_back(ho);
        ah->host_allocs.push_back(hb);
        ah->child_buffers[i] = {nullptr, ho, hb};
      } else if (c->type == DType::Utf8) {
        int32_t* ho = static_cast<int32_t*>(std::malloc(4));
        ho[0] = 0;
        char* hb = static_cast<char*>(std::malloc(1));
        ah->host_allocs.push_back(ho);
        ah->host_allocs.push_back(hb);
        ah->child_buffers[i] = {nullptr, ho, hb};
      } else {
        int64_t b = n * dtype_width(c->type);
        void* h = std::malloc(b > 0 ? b : 1);
        memcpy_d2h(h, c->data, b, s);
        ah->host_allocs.push_back(h);
        ah->child_buffers[i] = {nullptr, h};
      }
      if (c->valid != nullptr) {
        const int64_t vb = (n + 7) / 8;
        void* hv = std::malloc(vb > 0 ? vb : 1);
        memcpy_d2h(hv, c->valid, vb, s);
        ah->host_allocs.push_back(hv);
        ah->child_buffers[i][0] = hv;
      }
    }
    sync(s);
    ah->ts.reset();
  } else {
    for (int i = 0; i < nc; ++i) {
      const auto& c = ts->column(i);
      if (c->type == DType::Utf8)
        ah->child_buffers[i] = {c->valid, c->offsets, c->data};
      else
        ah->child_buffers[i] = {c->valid, c->data};
    }
  }
  for (int i = 0; i < nc; ++i) {
    ArrowArray& c = ah->child_structs[i];
    std::memset(&c, 0, sizeof(c));
    c.length = n;
    c.null_count = ah->child_buffers[i][0] != nullptr ? -1 : 0;  // -1: not counted
    c.offset = 0;
    c.n_buffers = static_cast<int64_t>(ah->child_buffers[i].size());
    c.buffers = ah->child_buffers[i].data();
    c.release = release_child_array;
    ah->child_ptrs[i] = &c;
  }
  ah->struct_buffers = {nullptr};
  std::memset(ao, 0, sizeof(*ao));
  ao->array.length = n;
  ao->array.null_count = 0;
  ao->array.offset = 0;
  ao->array.n_buffers = 1;
  ao->array.buffers = ah->struct_buffers.data();
  ao->array.n_children = nc;
  ao->array.children = nc > 0 ? ah->child_ptrs.data() : nullptr;
  ao->array.release = release_array;
  ao->array.private_data = ah;
  ao->device_type = to_host ? ARROW_DEVICE_CPU : ARROW_DEVICE_CUDA;
  ao->device_id = to_host ? -1 : current_device();
  ao->sync_event = nullptr;
}

void export_host_columns(const std::vector<Field>& fields, int64_t n,
                         const std::vector<std::vector<const void*>>& bufs, ArrowSchema* so, ArrowDeviceArray* ao) {
  const int nc = static_cast<int>(fields.size());
  auto* sh = new SchemaHolder();
  sh->names.reserve(nc);
  sh->child_structs.resize(nc);
  sh->child_ptrs.resize(nc);
  for (int i = 0; i < nc; ++i) {
    sh->names.push_back(fields[i].name);
    ArrowSchema& c = sh->child_structs[i];
    std::memset(&c, 0, sizeof(c));
    c.format = dtype_format(fields[i].type);
    c.name = sh->names.back().c_str();
    c.release = release_child_schema;
    sh->child_ptrs[i] = &c;
  }
  std::memset(so, 0, sizeof(*so));
  so->format = "+s";
  so->name = "";
  so->n_children = nc;
  so->children = nc > 0 ? sh->child_ptrs.data() : nullptr;
  so->release = release_schema;
  so->private_data = sh;

  auto* ah = new ArrayHolder();
  ah->child_structs.resize(nc);
  ah->child_ptrs.resize(nc);
  ah->child_buffers.resize(nc);
  for (int i = 0; i < nc; ++i) {
    if (fields[i].type == DType::Utf8) {
      const int32_t* offs = static_cast<const int32_t*>(bufs[i][0]);
      const char* bytes = static_cast<const char*>(bufs[i][1]);
      const int32_t first = n > 0 ? offs[0] : 0, last = n > 0 ? offs[n] : 0;
      auto* ho = static_cast<int32_t*>(std::malloc((n + 1) * 4));
      char* hb = static_cast<char*>(std::malloc(last - first > 0 ? last - first : 1));
      for (int64_t k = 0; k <= n; ++k) ho[k] = n > 0 ? offs[k] - first : 0;
      if (last > first) std::memcpy(hb, bytes + first, last - first);
      ah->host_allocs.push_back(ho);
      ah->host_allocs.push_back(hb);
      ah->child_buffers[i] = {nullptr, ho, hb};
    } else {
      const int64_t b = n * dtype_width(fields[i].type);
      void* h = std::malloc(b > 0 ? b : 1);
      if (b > 0) std::memcpy(h, bufs[i][0], b);
      ah->host_allocs.push_back(h);
      ah->child_buffers[i] = {nullptr, h};
    }
    ArrowArray& c = ah->child_structs[i];
    std::memset(&c, 0, sizeof(c));
    c.length = n;
    c.n_buffers = static_cast<int64_t>(ah->child_buffers[i].size());
    c.buffers = ah->child_buffers[i].data();
    c.release = release_child_array;
    ah->child_ptrs[i] = &c;
  }
  ah->struct_buffers = {nullptr};
  std::memset(ao, 0, sizeof(*ao));
  ao->array.length = n;
  ao->array.n_buffers = 1;
  ao->array.buffers = ah->struct_buffers.data();
  ao->array.n_children = nc;
  ao->array.children = nc > 0 ? ah->child_ptrs.data() : nullptr;
  ao->array.release = release_array;
  ao->array.private_data = ah;
  ao->device_type = ARROW_DEVICE_CPU;
  ao->device_id = -1;
}

}  // namespace gfpdb
