#include "pop.h"

#include <algorithm>
#include <cstdio>
#include <cstring>

namespace gfpdb::pop {

const char* message_type_name(MessageType t) {
  switch (t) {
    case MessageType::START: return "START";
    case MessageType::TUPLESET: return "TUPLESET";
    case MessageType::BLOOM_FILTER: return "BLOOM_FILTER";
    case MessageType::COMPLETE: return "COMPLETE";
    case MessageType::ERROR: return "ERROR";
  }
  return "?";
}

// ------------------------------------------------------- LocalPOpDirectory

void LocalPOpDirectory::add(const std::string& name, POpRelationshipType rel) { entries_[name].rels.insert(rel); }

void LocalPOpDirectory::setComplete(const std::string& name) {
  auto it = entries_.find(name);
  if (it != entries_.end()) it->second.complete = true;
}

bool LocalPOpDirectory::isComplete(const std::string& name) const {
  auto it = entries_.find(name);
  return it != entries_.end() && it->second.complete;
}

bool LocalPOpDirectory::allComplete(POpRelationshipType rel) const {
  for (auto& kv : entries_)
    if (kv.second.rels.count(rel) && !kv.second.complete) return false;
  return true;
}

bool LocalPOpDirectory::has(const std::string& name, POpRelationshipType rel) const {
  auto it = entries_.find(name);
  return it != entries_.end() && it->second.rels.count(rel) > 0;
}

std::vector<std::string> LocalPOpDirectory::names(POpRelationshipType rel) const {
  std::vector<std::string> out;
  for (auto& kv : entries_)
    if (kv.second.rels.count(rel)) out.push_back(kv.first);
  return out;
}

// -------------------------------------------------------------- POpContext

void POpContext::tell(Message msg) { tell(std::move(msg), op_->consumers()); }

void POpContext::tell(Message msg, const std::vector<std::string>& consumers) {
  msg.sender = op_->name();
  exec_->stamp(msg, op_);
  for (auto& c : consumers) exec_->post(c, msg);
}

void POpContext::notifyComplete() {
  if (complete_) return;
  complete_ = true;
  Message m;
  m.type = MessageType::COMPLETE;
  tell(m);
  exec_->markComplete(op_->name());
  op_->clear();
}

void POpContext::notifyError(const std::string& error) { exec_->error(op_->name(), error); }

LocalPOpDirectory& POpContext::operatorMap() { return op_->directory(); }

cudaStream_t POpContext::stream() const { return exec_->streamOf(op_); }

cudaStream_t POpContext::sideStream(int k) const { return exec_->sideStreamOf(op_, k); }

void POpContext::streamWait(cudaStream_t waiter, cudaStream_t on) { exec_->streamWait(waiter, on); }

// ------------------------------------------------------------------ ops

namespace {

bool is_producer_complete(PhysicalOp& op) { return op.ctx()->operatorMap().allComplete(POpRelationshipType::Producer); }

// Emits an input table (FileScanAbstractPOp::readAndSendTuples,
// fpdb-executor/src/physical/file/FileScanAbstractPOp.cpp:73-130, reading a
// table the caller handed over instead of a file), optionally split into
// zero-copy row slices.
class TableScanPOp : public PhysicalOp {
 public:
  TableScanPOp(std::string name, std::string table, std::vector<std::string> columns, int64_t chunk_rows,
               std::vector<std::string> in_place = {})
      : PhysicalOp(std::move(name), "TableScanPOp"), table_(std::move(table)), columns_(std::move(columns)),
        in_place_(std::move(in_place)), chunk_rows_(chunk_rows) {}

  void setExecution(Execution* e) { exec_ = e; }

  void onReceive(const Envelope& env) override {
    const Message& m = env.getMessage();
    if (m.type != MessageType::START) return;
    const InputTable& in = exec_->input(table_);
    // host tables: only the scanned columns come over, those named in
    // inPlaceColumns read in place when the table is page-locked
    TupleSetPtr ts = in.device ? in.device
                               : import_tupleset(in.schema, in.array, ctx()->stream(), false,
                                                 columns_.empty() ? nullptr : &columns_, &in_place_);
    if (!columns_.empty()) ts = ts->project(columns_);
    const int64_t n = ts->num_rows();
    if (chunk_rows_ <= 0 || n <= chunk_rows_) {
      send(ts);
    } else {
      for (int64_t at = 0; at < n; at += chunk_rows_) send(slice(ts, at, std::min(chunk_rows_, n - at)));
    }
    ctx()->notifyComplete();
  }

 private:
  static TupleSetPtr slice(const TupleSetPtr& ts, int64_t at, int64_t len) { return slice_rows(ts, at, len); }
  void send(const TupleSetPtr& ts) {
    Message out;
    out.type = MessageType::TUPLESET;
    out.tuples = ts;
    ctx()->tell(out);
  }

  Execution* exec_ = nullptr;
  std::string table_;
  std::vector<std::string> columns_;
  std::vector<std::string> in_place_;
  int64_t chunk_rows_;
};

// FilterPOp (fpdb-executor/src/physical/filter/FilterPOp.cpp:83-138,297-339,
// 475-482): predicate compiled once against the first TupleSet's schema
// (buildFilter), each TupleSet filtered and projected on the device.
class FilterPOp : public PhysicalOp {
 public:
  FilterPOp(std::string name, ExprPtr predicate) : PhysicalOp(std::move(name), "FilterPOp"), pred_(std::move(predicate)) {}

  void onReceive(const Envelope& env) override {
    const Message& m = env.getMessage();
    if (m.type == MessageType::TUPLESET) {
      const TupleSet& ts = *m.tuples;
      if (!compiled_) {
        // checkApplicability (FilterPOp.cpp:638-646): predicate columns must exist.
        compiled_.reset(new CompiledPredicate(compile_predicate(pred_, ts.fields())));
      }
      std::vector<std::string> proj;
      bool all = projectColumnNames_.empty();
      if (!all)
        for (auto& c : projectColumnNames_)
          if (ts.column_index(c) >= 0) proj.push_back(c);
      Message out;
      out.type = MessageType::TUPLESET;
      out.tuples = select_rows(ts, compiled_.get(), {}, proj, all, ctx()->stream());
      ctx()->tell(out);
    } else if (m.type == MessageType::COMPLETE) {
      if (is_producer_complete(*this)) ctx()->notifyComplete();
    }
  }

  void clear() override { compiled_.reset(); }

 private:
  ExprPtr pred_;
  std::unique_ptr<CompiledPredicate> compiled_;
};

// BloomFilterCreatePOp (fpdb-executor/src/physical/bloomfilter/BloomFilterCreatePOp.cpp:18-137):
// forwards every TupleSet to its ordinary consumers, keeps the key columns,
// and once all producers are complete builds the filter on the device and
// sends it to the BloomFilterUsePOps.
//
// The ordinary consumers are every consumer that is not a filter receiver,
// or, when the plan lists them ("dataConsumers", which the pipeline fusion
// writes once a join may both take this operator's rows and receive its
// filter), exactly those.
//
// After pipeline fusion (fuse_creator_chains) one operator may build several
// filters over the same rows, each on its own column for its own receivers,
// in one pass (bloom_build_many); each filter's messages name the creator
// it came from ("origin"), which its receivers know it by.
struct CreatedFilter {
  std::string origin;  // the creator's name in the unfused plan
  std::string column;
  int bits = 10, hashes = 3;
  std::vector<std::string> uses;
};

class BloomFilterCreatePOp : public PhysicalOp {
 public:
  BloomFilterCreatePOp(std::string name, std::vector<CreatedFilter> filters,
                       std::optional<std::vector<std::string>> data_consumers = std::nullopt)
      : PhysicalOp(std::move(name), "BloomFilterCreatePOp"), filters_(std::move(filters)),
        data_consumers_(std::move(data_consumers)) {
    if (filters_.empty() || filters_.size() > static_cast<size_t>(kBloomBuildManyMax))
      fail(GFPDB_EINVAL, "BloomFilterCreatePOp '" + name_ + "': 1 to 8 filters");
    for (auto& f : filters_)
      for (auto& u : f.uses)
        if (std::find(uses_.begin(), uses_.end(), u) == uses_.end()) uses_.push_back(u);
  }

  void onReceive(const Envelope& env) override {
    const Message& m = env.getMessage();
    if (m.type == MessageType::TUPLESET) {
      for (auto& f : filters_) m.tuples->require_column(f.column);
      buffered_.push_back(m.tuples);
      std::vector<std::string> pass;
      if (data_consumers_)
        pass = *data_consumers_;
      else
        for (auto& c : consumers_)
          if (std::find(uses_.begin(), uses_.end(), c) == uses_.end()) pass.push_back(c);
      Message out;
      out.type = MessageType::TUPLESET;
      out.tuples = m.tuples;
      ctx()->tell(out, pass);
    } else if (m.type == MessageType::COMPLETE) {
      if (!is_producer_complete(*this)) return;
      std::vector<const int64_t*> rows;
      std::vector<std::vector<const Column*>> parts(filters_.size());
      std::vector<int32_t> bits, hashes;
      for (auto& t : buffered_) rows.push_back(t->rows_dev());
      for (size_t f = 0; f < filters_.size(); ++f) {
        for (auto& t : buffered_) parts[f].push_back(t->column(filters_[f].column).get());
        bits.push_back(filters_[f].bits);
        hashes.push_back(filters_[f].hashes);
      }
      std::vector<BloomPtr> blooms;
      if (filters_.size() == 1)
        blooms.push_back(bloom_build(parts[0], bits[0], hashes[0], ctx()->stream(), rows));
      else
        blooms = bloom_build_many(parts, bits, hashes, ctx()->stream(), rows);
      for (size_t f = 0; f < filters_.size(); ++f) {
        Message out;
        out.type = MessageType::BLOOM_FILTER;
        out.bloom = blooms[f];
        if (filters_[f].origin != name_) out.origin = filters_[f].origin;
        ctx()->tell(out, filters_[f].uses);
      }
      ctx()->notifyComplete();
    }
  }

  void clear() override { buffered_.clear(); }

 private:
  std::vector<CreatedFilter> filters_;
  std::vector<std::string> uses_;  // every filter's receivers
  std::optional<std::vector<std::string>> data_consumers_;
  std::vector<TupleSetPtr> buffered_;
};

// BloomFilterUsePOp (fpdb-executor/src/physical/bloomfilter/BloomFilterUsePOp.cpp:71-142):
// buffers TupleSets until the filter arrives, then filters each one.
//
// After pipeline fusion (fuse_bloom_chains below) one BloomFilterUsePOp may
// carry several (column, creator) probes: it waits for every filter and then
// applies them all in one pass over each TupleSet, in chain order.
class BloomFilterUsePOp : public PhysicalOp {
 public:
  BloomFilterUsePOp(std::string name, std::vector<std::string> columns, std::vector<std::string> creators)
      : PhysicalOp(std::move(name), "BloomFilterUsePOp"), columns_(std::move(columns)),
        creators_(std::move(creators)), blooms_(columns_.size()) {}

  void onReceive(const Envelope& env) override {
    const Message& m = env.getMessage();
    if (m.type == MessageType::TUPLESET) {
      if (ready()) filterAndSend(m.tuples);
      else buffered_.push_back(m.tuples);
    } else if (m.type == MessageType::BLOOM_FILTER) {
      size_t i = 0;
      if (!creators_.empty()) {
        const std::string& from = m.origin.empty() ? m.sender : m.origin;
        auto it = std::find(creators_.begin(), creators_.end(), from);
        if (it == creators_.end()) fail(GFPDB_EINVAL, "BloomFilterUsePOp '" + name_ + "': filter from '" + from + "'");
        i = static_cast<size_t>(it - creators_.begin());
      }
      blooms_[i] = m.bloom;
      if (ready()) {
        for (auto& t : buffered_) filterAndSend(t);
        buffered_.clear();
      }
    } else if (m.type == MessageType::COMPLETE) {
      if (!is_producer_complete(*this)) return;
      if (!ready() && !buffered_.empty())
        fail(GFPDB_EINVAL, "BloomFilterUsePOp '" + name_ + "': producers completed without a bloom filter");
      ctx()->notifyComplete();
    }
  }

  void clear() override {
    buffered_.clear();
    for (auto& b : blooms_) b.reset();
  }

 private:
  bool ready() const {
    for (auto& b : blooms_)
      if (!b) return false;
    return true;
  }
  void filterAndSend(const TupleSetPtr& ts) {
    std::vector<BloomProbe> probes;
    for (size_t i = 0; i < columns_.size(); ++i) probes.push_back(BloomProbe{blooms_[i], columns_[i]});
    Message out;
    out.type = MessageType::TUPLESET;
    out.tuples = select_rows(*ts, nullptr, probes, {}, true, ctx()->stream());
    ctx()->tell(out);
  }
  std::vector<std::string> columns_;
  std::vector<std::string> creators_;
  std::vector<BloomPtr> blooms_;
  std::vector<TupleSetPtr> buffered_;
};

// One hash join's probe of one TupleSet (the output: probe fields then build
// fields, HashJoinArrowKernel.cpp:148-162, each kept when projected).
TupleSetPtr probe_join(const std::string& join_name, const JoinTable& table, const std::vector<std::string>& proj,
                       const std::string& probe_key, const TupleSetPtr& ts, cudaStream_t stream) {
  const int pk = ts->require_column(probe_key);
  auto needed = [&](const std::string& c) {
    return proj.empty() ||
           std::find(proj.begin(), proj.end(), c) != proj.end();
  };
  // Output: probe fields then build fields (HashJoinArrowKernel.cpp:148-162),
  // each filtered to the needed columns.
  {
    std::vector<Field> fields;
    std::vector<int> pcols, bcols;
    bool fixed = true;
    for (int i = 0; i < ts->num_columns(); ++i)
      if (needed(ts->field(i).name)) {
        fields.push_back(ts->field(i));
        pcols.push_back(i);
        fixed &= ts->field(i).type != DType::Utf8;
      }
    const TupleSet& b = *table.build;
    for (int i = 0; i < b.num_columns(); ++i)
      if (needed(b.field(i).name)) {
        for (auto& f : fields)
          if (f.name == b.field(i).name)
            fail(GFPDB_EINVAL, "HashJoinArrowPOp '" + join_name + "': column '" + f.name + "' is on both sides");
        fields.push_back(b.field(i));
        bcols.push_back(i);
        fixed &= b.field(i).type != DType::Utf8;
      }
    if (fixed) {
      // fixed-width outputs: probe and materialise in one kernel
      BufferPtr count_owner;
      const int64_t* count_dev = nullptr;
      int64_t n = 0;
      auto cols = join_probe_materialize(table, *ts, pk, pcols, bcols, &n, stream, &count_owner,
                                         &count_dev);
      if (count_dev != nullptr)
        return TupleSet::make_deferred(std::move(fields), std::move(cols), n, count_owner, count_dev);
      return TupleSet::make(std::move(fields), std::move(cols), n);
    }
  }
  BufferPtr pidx, bidx, count_owner;
  const int64_t* count_dev = nullptr;
  int64_t n = 0;
  join_probe_pairs(table, *ts, pk, &pidx, &bidx, &n, stream, &count_owner, &count_dev);
  std::vector<GatherSpec> specs;
  std::vector<Field> fields;
  for (int i = 0; i < ts->num_columns(); ++i)
    if (needed(ts->field(i).name)) {
      fields.push_back(ts->field(i));
      specs.push_back(GatherSpec{ts->column(i).get(), pidx->as<int32_t>()});
    }
  const TupleSet& b = *table.build;
  for (int i = 0; i < b.num_columns(); ++i)
    if (needed(b.field(i).name)) {
      for (auto& f : fields)
        if (f.name == b.field(i).name)
          fail(GFPDB_EINVAL, "HashJoinArrowPOp '" + join_name + "': column '" + f.name + "' is on both sides");
      fields.push_back(b.field(i));
      specs.push_back(GatherSpec{b.column(i).get(), bidx->as<int32_t>()});
    }
  bool utf8 = false;
  for (auto& f : fields) utf8 |= f.type == DType::Utf8;
  if (count_dev != nullptr && utf8) {
    // utf8 outputs are sized from the exact pair count
    int64_t exact = 0;
    GF_CUDA(cudaMemcpyAsync(&exact, count_dev, sizeof(exact), cudaMemcpyDeviceToHost, stream));
    sync(stream);
    n = exact < n ? exact : n;
    count_dev = nullptr;
  }
  auto cols = gather_columns(specs, n, stream, count_dev, count_owner);
  if (count_dev != nullptr)
    return TupleSet::make_deferred(std::move(fields), std::move(cols), n, count_owner, count_dev);
  return TupleSet::make(std::move(fields), std::move(cols), n);
}

}  // namespace

TupleSetPtr filter_build_side(const TupleSetPtr& build, const std::string& key, const std::vector<BloomProbe>& filters,
                              cudaStream_t s, std::vector<BloomPtr>* in_build) {
  in_build->clear();
  if (filters.empty()) return build;
  bool on_key = !key.empty() && filters.size() <= static_cast<size_t>(kJoinBuildFiltersMax);
  if (on_key) {
    const DType kt = build->field(build->require_column(key)).type;
    on_key = kt == DType::Int32 || kt == DType::Int64 || kt == DType::Date32;
  }
  for (auto& f : filters) on_key &= f.column == key;
  if (on_key) {
    for (auto& f : filters) in_build->push_back(f.bloom);
    return build;
  }
  return select_rows(*build, nullptr, filters, {}, true, s);
}

// The join table over a build side: keyed on its single key column, or on
// the composite of several (with the key columns aliased for the equality
// check that probe_join_multi makes).
JoinTable build_join_table(const TupleSetPtr& build_in, const std::vector<std::string>& keys, double load_factor,
                           cudaStream_t s, bool mark, const std::vector<BloomProbe>& filters) {
  JoinTable t;
  std::vector<BloomPtr> in_build;
  TupleSetPtr build = filter_build_side(build_in, keys.size() == 1 && !mark ? keys[0] : std::string(), filters, s,
                                        &in_build);
  // A marking join reads its build rows' flags back by row (the rows of an
  // outer join that no probe row matched): its build side needs its exact
  // row count, not a device-sized capacity.
  if (mark) build = resolved(build, s);
  // a utf8 key, like several key columns, is joined on its hash and checked
  // on the key itself
  t.composite = keys.size() > 1 || build->field(build->require_column(keys[0])).type == DType::Utf8;
  t.build = t.composite ? with_composite_key(build, keys, kBuildKeyColumn, kBuildKeyAlias, s) : build;
  t.key_col = t.build->require_column(t.composite ? std::string(kBuildKeyColumn) : keys[0]);
  join_build_table(t, load_factor, s, in_build);
  if (mark) {
    if (t.composite)
      fail(GFPDB_EUNSUPPORTED, "outer and semi joins take one integer key column per side");
    t.matched = make_filled((t.build->num_rows() > 0 ? t.build->num_rows() : 1) * 4, 0, s);
  }
  return t;
}

namespace {

// A join on several key columns (HashJoinPredicate's column lists,
// fpdb-executor/include/fpdb/executor/physical/join/hashjoin/HashJoinPredicate.h:25-26),
// over a table built on the build side's composite key (with its key columns
// aliased, build_join_table): the probe side gets its composite, the join
// pairs composites, and a selection keeps the rows whose key columns are
// equal pairwise, so composite collisions cannot add rows. The output is the
// single-key join's: probe then build columns, filtered to `proj`.
TupleSetPtr probe_join_multi(const std::string& join_name, const JoinTable& table,
                             const std::vector<std::string>& proj, const std::vector<std::string>& probe_keys,
                             const TupleSetPtr& ts, cudaStream_t stream) {
  TupleSetPtr pk = with_composite_key(ts, probe_keys, kProbeKeyColumn, "", stream);
  const TupleSet& b = *table.build;
  std::vector<std::string> wanted;  // requested output columns
  if (proj.empty()) {
    for (int i = 0; i < ts->num_columns(); ++i) wanted.push_back(ts->field(i).name);
    for (int i = 0; i < b.num_columns(); ++i)
      if (!is_internal_key_column(b.field(i).name)) wanted.push_back(b.field(i).name);
  } else {
    wanted = proj;
  }
  std::vector<std::string> with_keys = wanted;
  for (const auto& k : probe_keys)
    if (std::find(with_keys.begin(), with_keys.end(), k) == with_keys.end()) with_keys.push_back(k);
  for (size_t i = 0; i < probe_keys.size(); ++i) with_keys.push_back(kBuildKeyAlias + std::to_string(i));
  TupleSetPtr joined = probe_join(join_name, table, with_keys, kProbeKeyColumn, pk, stream);
  auto conj = std::make_shared<Expr>();
  conj->kind = Expr::And;
  for (size_t i = 0; i < probe_keys.size(); ++i) {
    auto l = std::make_shared<Expr>();
    l->kind = Expr::Column;
    l->name = probe_keys[i];
    auto r = std::make_shared<Expr>();
    r->kind = Expr::Column;
    r->name = kBuildKeyAlias + std::to_string(i);
    auto eq = std::make_shared<Expr>();
    eq->kind = Expr::Compare;
    eq->cmp = LO_EQ;
    eq->kids = {l, r};
    conj->kids.push_back(eq);
  }
  const CompiledPredicate pred = compile_predicate(conj, joined->fields());
  std::vector<std::string> out_cols;  // the join's order (probe, then build) of the requested columns
  for (int i = 0; i < joined->num_columns(); ++i) {
    const std::string& n = joined->field(i).name;
    if (std::find(wanted.begin(), wanted.end(), n) != wanted.end()) out_cols.push_back(n);
  }
  return select_rows(*joined, &pred, {}, out_cols, false, stream);
}

}  // namespace

TupleSetPtr join_probe_keys(const std::string& join_name, const JoinTable& table, const std::vector<std::string>& proj,
                            const std::vector<std::string>& probe_keys, const TupleSetPtr& ts, cudaStream_t s) {
  return !table.composite ? probe_join(join_name, table, proj, probe_keys[0], ts, s)
                          : probe_join_multi(join_name, table, proj, probe_keys, ts, s);
}

JoinKind join_kind_from_name(const std::string& name) {
  if (name == "INNER") return JoinKind::Inner;
  if (name == "LEFT") return JoinKind::Left;
  if (name == "RIGHT") return JoinKind::Right;
  if (name == "FULL") return JoinKind::Full;
  if (name == "LEFT_SEMI") return JoinKind::LeftSemi;
  if (name == "RIGHT_SEMI") return JoinKind::RightSemi;
  fail(GFPDB_EINVAL, "join type '" + name + "' (INNER, LEFT, RIGHT, FULL, LEFT_SEMI or RIGHT_SEMI)");
}

bool join_kind_marks(JoinKind k) { return k == JoinKind::Left || k == JoinKind::Full || k == JoinKind::LeftSemi; }

namespace {

bool wanted(const std::vector<std::string>& proj, const std::string& c) {
  return proj.empty() || std::find(proj.begin(), proj.end(), c) != proj.end();
}

// The join's output columns of one side: (field, source column index).
std::vector<std::pair<Field, int>> side_columns(const std::vector<Field>& fields, const std::vector<std::string>& proj) {
  std::vector<std::pair<Field, int>> out;
  for (size_t i = 0; i < fields.size(); ++i)
    if (!is_internal_key_column(fields[i].name) && wanted(proj, fields[i].name))
      out.emplace_back(fields[i], static_cast<int>(i));
  return out;
}

// Gathers probe columns by pidx and build columns by bidx (either may be
// null: that side left out), the build side's indexes possibly -1 (nulls).
TupleSetPtr join_gather(const std::string& join_name, const TupleSet* probe, const BufferPtr& pidx,
                        const TupleSet& build, const BufferPtr& bidx, bool build_nulls,
                        const std::vector<std::string>& proj, int64_t n, cudaStream_t s) {
  std::vector<Field> fields;
  std::vector<GatherSpec> specs;
  if (probe != nullptr)
    for (auto& [f, i] : side_columns(probe->fields(), proj)) {
      fields.push_back(f);
      specs.push_back(GatherSpec{probe->column(i).get(), pidx->as<int32_t>(), false});
    }
  if (bidx)
    for (auto& [f, i] : side_columns(build.fields(), proj)) {
      for (auto& g : fields)
        if (g.name == f.name)
          fail(GFPDB_EINVAL, "HashJoinArrowPOp '" + join_name + "': column '" + f.name + "' is on both sides");
      fields.push_back(f);
      specs.push_back(GatherSpec{build.column(i).get(), bidx->as<int32_t>(), build_nulls});
    }
  return TupleSet::make(std::move(fields), gather_columns(specs, n, s), n);
}

}  // namespace

TupleSetPtr join_probe_kind(const std::string& join_name, JoinKind kind, const JoinTable& table,
                            const std::vector<std::string>& proj, const std::vector<std::string>& probe_keys,
                            const TupleSetPtr& in, cudaStream_t s) {
  if (kind == JoinKind::Inner) return join_probe_keys(join_name, table, proj, probe_keys, in, s);
  if (table.composite) fail(GFPDB_EUNSUPPORTED, "outer and semi joins take one integer key column per side");
  TupleSetPtr ts = resolved(in, s);
  const int pk = ts->require_column(probe_keys[0]);
  int32_t* matched = table.matched ? table.matched->as<int32_t>() : nullptr;
  BufferPtr pidx, bidx;
  int64_t n = 0;
  switch (kind) {
    case JoinKind::Right:  // every probe row, unmatched ones with a null build side
    case JoinKind::Full:
      join_pairs_ordered(table, *ts, pk, true, matched, &pidx, &bidx, &n, s);
      return join_gather(join_name, ts.get(), pidx, *table.build, bidx, true, proj, n, s);
    case JoinKind::Left:  // the matches now, the unmatched build rows at the end
      join_pairs_ordered(table, *ts, pk, false, matched, &pidx, &bidx, &n, s);
      return join_gather(join_name, ts.get(), pidx, *table.build, bidx, false, proj, n, s);
    case JoinKind::LeftSemi:  // build rows, emitted at the end
      join_match(table, *ts, pk, nullptr, false, matched, s);
      return nullptr;
    case JoinKind::RightSemi: {  // each probe row with a match, once
      auto counts = make_buffer((ts->num_rows() > 0 ? ts->num_rows() : 1) * 4, s);
      join_match(table, *ts, pk, counts->as<int32_t>(), false, nullptr, s);
      pidx = rows_where(counts->as<int32_t>(), ts->num_rows(), true, &n, s);
      return join_gather(join_name, ts.get(), pidx, *table.build, nullptr, false, proj, n, s);
    }
    default:
      break;
  }
  fail(GFPDB_EINVAL, "unknown join kind");
}

TupleSetPtr join_finish_kind(const std::string& join_name, JoinKind kind, const JoinTable& table,
                             const std::vector<Field>& probe_fields, const std::vector<std::string>& proj,
                             cudaStream_t s) {
  if (!join_kind_marks(kind)) return nullptr;
  const int64_t nb = table.build->num_rows();
  int64_t n = 0;
  BufferPtr rows = rows_where(table.matched->as<int32_t>(), nb, kind == JoinKind::LeftSemi, &n, s);
  if (kind == JoinKind::LeftSemi)
    return join_gather(join_name, nullptr, nullptr, *table.build, rows, false, proj, n, s);
  // unmatched build rows, their probe columns null
  TupleSetPtr b = join_gather(join_name, nullptr, nullptr, *table.build, rows, false, proj, n, s);
  std::vector<Field> fields;
  std::vector<ColumnPtr> cols;
  for (auto& [f, i] : side_columns(probe_fields, proj)) {
    (void)i;
    fields.push_back(f);
    cols.push_back(null_column(f.type, n, s));
  }
  for (int i = 0; i < b->num_columns(); ++i) {
    fields.push_back(b->field(i));
    cols.push_back(b->column(i));
  }
  return TupleSet::make(std::move(fields), std::move(cols), n);
}

namespace {

// The bloom filters a join build tests (predicate transfer's backward
// filters on a dimension, moved into the join by the plan's pipeline fusion,
// fuse_build_filters): per filter the build column it tests and the
// BloomFilterCreatePOp that sends it.
struct BuildFilterSpec {
  std::vector<std::string> columns, creators;
  std::vector<BloomPtr> blooms;

  static const std::string& origin_of(const Message& m) { return m.origin.empty() ? m.sender : m.origin; }
  bool takes(const Message& m) const {
    return std::find(creators.begin(), creators.end(), origin_of(m)) != creators.end();
  }
  void receive(const std::string& op, const Message& m) {
    auto it = std::find(creators.begin(), creators.end(), origin_of(m));
    if (it == creators.end()) fail(GFPDB_EINVAL, "HashJoinArrowPOp '" + op + "': bloom filter from '" + origin_of(m) + "'");
    blooms[static_cast<size_t>(it - creators.begin())] = m.bloom;
  }
  bool ready() const {
    for (auto& b : blooms)
      if (!b) return false;
    return true;
  }
  void require_all(const std::string& op) const {
    if (!ready()) fail(GFPDB_EINVAL, "HashJoinArrowPOp '" + op + "': producers completed without its bloom filters");
  }
  std::vector<BloomProbe> probes() const {
    std::vector<BloomProbe> p;
    for (size_t i = 0; i < columns.size(); ++i) p.push_back(BloomProbe{blooms[i], columns[i]});
    return p;
  }
  void reset() {
    for (auto& b : blooms) b.reset();
  }
};

// "buildFilters": [{"column": c, "creator": op}, ...]
BuildFilterSpec parse_build_filters(const json::Value& o) {
  BuildFilterSpec f;
  if (!o.contains("buildFilters")) return f;
  for (auto& e : o.at("buildFilters").array()) {
    f.columns.push_back(e.at("column").str());
    f.creators.push_back(e.at("creator").str());
  }
  f.blooms.resize(f.columns.size());
  return f;
}

// HashJoinArrowPOp (fpdb-executor/src/physical/join/hashjoin/HashJoinArrowPOp.cpp:85-153):
// routes TupleSets by sender to the build or probe side, builds the table
// once every build producer is complete, probes as probe input arrives.
class HashJoinArrowPOp : public PhysicalOp {
 public:
  HashJoinArrowPOp(std::string name, std::vector<std::string> build_producers, std::vector<std::string> probe_producers,
                   std::vector<std::string> build_keys, std::vector<std::string> probe_keys, double load_factor,
                   JoinKind kind = JoinKind::Inner, BuildFilterSpec filters = {})
      : PhysicalOp(std::move(name), "HashJoinArrowPOp"), build_producers_(std::move(build_producers)),
        probe_producers_(std::move(probe_producers)), build_keys_(std::move(build_keys)),
        probe_keys_(std::move(probe_keys)), load_factor_(load_factor), kind_(kind), filters_(std::move(filters)) {
    if (build_keys_.empty() || build_keys_.size() != probe_keys_.size())
      fail(GFPDB_EINVAL, "HashJoinArrowPOp '" + name_ + "': as many probe keys as build keys, at least one");
  }

  void onReceive(const Envelope& env) override {
    const Message& m = env.getMessage();
    if (m.type == MessageType::TUPLESET) {
      if (is_build(m.sender)) {
        if (built_) fail(GFPDB_EINVAL, "HashJoinArrowPOp '" + name_ + "': build input after the table was built");
        build_.push_back(m.tuples);
      } else {
        if (built_) probe(m.tuples);
        else probe_buffer_.push_back(m.tuples);
      }
    } else if (m.type == MessageType::BLOOM_FILTER) {
      filters_.receive(name_, m);
      maybeBuild();
    } else if (m.type == MessageType::COMPLETE) {
      maybeBuild();
      if (is_producer_complete(*this)) {
        if (!built_) {
          filters_.require_all(name_);
          finalizeBuild();
        }
        // outer and semi joins: the build rows decided once every probe row is in
        Message out;
        out.type = MessageType::TUPLESET;
        out.tuples = join_finish_kind(name_, kind_, table_, probe_fields_, projectColumnNames_, ctx()->stream());
        if (out.tuples) ctx()->tell(out);
        ctx()->notifyComplete();
      }
    }
  }

  void clear() override {
    build_.clear();
    probe_buffer_.clear();
    table_ = JoinTable{};
    built_ = false;
    filters_.reset();
  }

 private:
  bool is_build(const std::string& sender) const {
    return std::find(build_producers_.begin(), build_producers_.end(), sender) != build_producers_.end();
  }

  // The table is built once every build producer is complete and every
  // bloom filter the build tests has arrived; buffered probes follow.
  void maybeBuild() {
    if (built_ || !filters_.ready()) return;
    auto& dir = ctx()->operatorMap();
    for (auto& b : build_producers_)
      if (!dir.isComplete(b)) return;
    finalizeBuild();
    for (auto& t : probe_buffer_) probe(t);
    probe_buffer_.clear();
  }

  void finalizeBuild() {
    if (build_.empty()) fail(GFPDB_EINVAL, "HashJoinArrowPOp '" + name_ + "': no build-side input");
    table_ = build_join_table(TupleSet::concatenate(build_, ctx()->stream()), build_keys_, load_factor_,
                              ctx()->stream(), join_kind_marks(kind_), filters_.probes());
    build_.clear();
    built_ = true;
  }

  void probe(const TupleSetPtr& ts) {
    if (probe_fields_.empty()) probe_fields_ = ts->fields();
    Message out;
    out.type = MessageType::TUPLESET;
    out.tuples = join_probe_kind(name_, kind_, table_, projectColumnNames_, probe_keys_, ts, ctx()->stream());
    if (out.tuples) ctx()->tell(out);
  }

  std::vector<std::string> build_producers_, probe_producers_;
  std::vector<std::string> build_keys_, probe_keys_;
  double load_factor_;
  JoinKind kind_;
  BuildFilterSpec filters_;
  std::vector<TupleSetPtr> build_, probe_buffer_;
  std::vector<Field> probe_fields_;  // the probe side's schema (null columns of unmatched build rows)
  JoinTable table_;
  bool built_ = false;
};

// HashJoinChainPOp: a chain of HashJoinArrowPOps in which each join's only
// consumer is the next join and is its probe side (the star join: fact rows
// probing one dimension after another), produced by the plan's pipeline
// fusion (fuse_join_chains). Every join's table is built as its build side
// completes, as HashJoinArrowPOp does; each probe TupleSet then goes through
// all the joins in one kernel (join_chain_materialize) that writes only the
// last join's output columns, instead of one probe launch and one
// intermediate TupleSet per join. Column selection, names and errors are the
// unfused chain's; outputs with utf8 columns take the joins one at a time.
struct ChainJoinSpec {
  std::string name;
  std::vector<std::string> build_producers;
  std::string build_key, probe_key;
  double load_factor = 0.5;
  std::vector<std::string> proj;
  BuildFilterSpec filters;
};

class HashJoinChainPOp : public PhysicalOp {
 public:
  HashJoinChainPOp(std::string name, std::vector<ChainJoinSpec> joins)
      : PhysicalOp(std::move(name), "HashJoinChainPOp"), joins_(std::move(joins)), build_(joins_.size()),
        tables_(joins_.size()), built_(joins_.size(), false) {
    if (joins_.empty() || static_cast<int>(joins_.size()) > kJoinChainMax)
      fail(GFPDB_EINVAL, "HashJoinChainPOp '" + name_ + "': 1 to 6 joins");
  }

  void onReceive(const Envelope& env) override {
    const Message& m = env.getMessage();
    if (m.type == MessageType::TUPLESET) {
      bool build = false;
      for (size_t l = 0; l < joins_.size(); ++l) {
        const auto& bp = joins_[l].build_producers;
        if (std::find(bp.begin(), bp.end(), m.sender) == bp.end()) continue;
        if (built_[l])
          fail(GFPDB_EINVAL, "HashJoinArrowPOp '" + joins_[l].name + "': build input after the table was built");
        build_[l].push_back(m.tuples);
        build = true;
      }
      if (build) return;
      if (allBuilt()) process(m.tuples);
      else probe_buffer_.push_back(m.tuples);
    } else if (m.type == MessageType::BLOOM_FILTER) {
      bool taken = false;
      for (auto& J : joins_)
        if (J.filters.takes(m)) {
          J.filters.receive(J.name, m);
          taken = true;
        }
      if (!taken) fail(GFPDB_EINVAL, "HashJoinChainPOp '" + name_ + "': bloom filter from '" + m.sender + "'");
      advance();
    } else if (m.type == MessageType::COMPLETE) {
      advance();
      if (is_producer_complete(*this)) {
        joinBuilds();
        // The tables were allocated on the build streams and are freed there
        // when this operator clears: those frees must follow every probe
        // issued on this operator's stream.
        for (cudaStream_t bs : used_streams_) ctx()->streamWait(bs, ctx()->stream());
        used_streams_.clear();
        ctx()->notifyComplete();
      }
    }
  }

  void clear() override {
    build_streams_.clear();
    used_streams_.clear();
    for (auto& b : build_) b.clear();
    probe_buffer_.clear();
    for (auto& t : tables_) t = JoinTable{};
    for (auto& J : joins_) J.filters.reset();
  }

 private:
  bool allBuilt() const { return std::all_of(built_.begin(), built_.end(), [](bool b) { return b; }); }

  // Builds every table whose build side is complete and whose bloom filters
  // have arrived (all of them once every producer is complete), then runs
  // the buffered probes when the last table is built.
  void advance() {
    auto& dir = ctx()->operatorMap();
    const bool all_done = is_producer_complete(*this);
    for (size_t l = 0; l < joins_.size(); ++l) {
      if (built_[l]) continue;
      if (all_done) joins_[l].filters.require_all(joins_[l].name);
      if (!joins_[l].filters.ready()) continue;
      bool done = true;
      for (auto& b : joins_[l].build_producers) done &= dir.isComplete(b);
      if (done || all_done) finalizeBuild(l);
    }
    if (allBuilt()) {
      for (auto& t : probe_buffer_) process(t);
      probe_buffer_.clear();
    }
  }

  // Each join's table is built on a stream of its own (its inputs were
  // waited for on this operator's stream, which the build stream joins
  // first); the operator's stream waits for every build just before the
  // first probe, so the builds run side by side.
  void finalizeBuild(size_t l) {
    const auto& J = joins_[l];
    if (build_[l].empty()) fail(GFPDB_EINVAL, "HashJoinArrowPOp '" + J.name + "': no build-side input");
    cudaStream_t bs = ctx()->sideStream(static_cast<int>(l));
    ctx()->streamWait(bs, ctx()->stream());
    std::vector<BloomPtr> in_build;
    tables_[l].build = filter_build_side(TupleSet::concatenate(build_[l], bs), J.build_key, J.filters.probes(), bs,
                                         &in_build);
    tables_[l].key_col = tables_[l].build->require_column(J.build_key);
    join_build_table(tables_[l], J.load_factor, bs, in_build);
    build_streams_.push_back(bs);
    if (std::find(used_streams_.begin(), used_streams_.end(), bs) == used_streams_.end()) used_streams_.push_back(bs);
    build_[l].clear();
    built_[l] = true;
  }

  void joinBuilds() {
    for (cudaStream_t bs : build_streams_) ctx()->streamWait(ctx()->stream(), bs);
    build_streams_.clear();
  }

  void process(const TupleSetPtr& ts) {
    joinBuilds();
    // Follow the columns through the chain by name, as the joins one at a
    // time would see them: (source, column) of every join's probe key and of
    // the last join's outputs.
    struct Col {
      Field f;
      ChainRef ref;
    };
    std::vector<Col> cur;
    for (int i = 0; i < ts->num_columns(); ++i) cur.push_back(Col{ts->field(i), ChainRef{0, i}});
    std::vector<ChainRef> keys;
    for (size_t l = 0; l < joins_.size(); ++l) {
      const auto& J = joins_[l];
      auto k = std::find_if(cur.begin(), cur.end(), [&](const Col& c) { return c.f.name == J.probe_key; });
      if (k == cur.end()) fail(GFPDB_EINVAL, "column '" + J.probe_key + "' not found in TupleSet");
      keys.push_back(k->ref);
      auto needed = [&](const std::string& c) {
        return J.proj.empty() || std::find(J.proj.begin(), J.proj.end(), c) != J.proj.end();
      };
      std::vector<Col> next;
      for (auto& c : cur)
        if (needed(c.f.name)) next.push_back(c);
      const TupleSet& b = *tables_[l].build;
      for (int i = 0; i < b.num_columns(); ++i) {
        if (!needed(b.field(i).name)) continue;
        for (auto& c : next)
          if (c.f.name == b.field(i).name)
            fail(GFPDB_EINVAL, "HashJoinArrowPOp '" + J.name + "': column '" + c.f.name + "' is on both sides");
        next.push_back(Col{b.field(i), ChainRef{static_cast<int>(l) + 1, i}});
      }
      cur = std::move(next);
    }
    bool fixed = true;
    for (auto& c : cur) fixed &= c.f.type != DType::Utf8;
    Message out;
    out.type = MessageType::TUPLESET;
    if (fixed) {
      std::vector<const JoinTable*> tabs;
      for (auto& t : tables_) tabs.push_back(&t);
      std::vector<ChainRef> outs;
      std::vector<Field> fields;
      for (auto& c : cur) {
        outs.push_back(c.ref);
        fields.push_back(c.f);
      }
      BufferPtr count_owner;
      const int64_t* count_dev = nullptr;
      int64_t n = 0;
      auto cols = join_chain_materialize(tabs, *ts, keys, outs, &n, ctx()->stream(), &count_owner, &count_dev);
      out.tuples = count_dev != nullptr
                       ? TupleSet::make_deferred(std::move(fields), std::move(cols), n, count_owner, count_dev)
                       : TupleSet::make(std::move(fields), std::move(cols), n);
    } else {
      TupleSetPtr t = ts;
      for (size_t l = 0; l < joins_.size(); ++l)
        t = probe_join(joins_[l].name, tables_[l], joins_[l].proj, joins_[l].probe_key, t, ctx()->stream());
      out.tuples = t;
    }
    ctx()->tell(out);
  }

  std::vector<ChainJoinSpec> joins_;
  std::vector<std::vector<TupleSetPtr>> build_;
  std::vector<JoinTable> tables_;
  std::vector<bool> built_;
  std::vector<TupleSetPtr> probe_buffer_;
  std::vector<cudaStream_t> build_streams_;  // builds the operator's stream has not yet waited for
  std::vector<cudaStream_t> used_streams_;   // every stream a table was built on
};

// GroupPOp (fpdb-executor/src/physical/group/GroupPOp.cpp:14-85): group each
// TupleSet as it arrives, finalise when all producers are complete.
class GroupPOp : public PhysicalOp {
 public:
  GroupPOp(std::string name, std::vector<std::string> group_cols, std::vector<GroupAggregate> aggs, int64_t hint,
           std::string type = "GroupPOp")
      : PhysicalOp(std::move(name), std::move(type)) {
    table_ = group_table_create(group_cols, aggs, hint);
  }

  void onReceive(const Envelope& env) override {
    const Message& m = env.getMessage();
    if (m.type == MessageType::TUPLESET) {
      group_table_update(*table_, *m.tuples, ctx()->stream());
    } else if (m.type == MessageType::COMPLETE) {
      if (!is_producer_complete(*this)) return;
      Message out;
      out.type = MessageType::TUPLESET;
      out.tuples = group_table_finalize(*table_, ctx()->stream());
      if (!projectColumnNames_.empty()) out.tuples = out.tuples->project_exist(projectColumnNames_);
      ctx()->tell(out);
      ctx()->notifyComplete();
    }
  }

  void clear() override { table_.reset(); }

 private:
  std::shared_ptr<GroupTable> table_;
};

// ShufflePOp (fpdb-executor/src/physical/shuffle/ShufflePOp.cpp:91-172): every
// TupleSet it receives is hash-partitioned on the shuffle columns into one
// slot per consumer (slot i goes to the i-th consumer in the plan's order,
// the reference's consumerVec_), and the slots are buffered. Once all
// producers are complete, each consumer gets its slot's rows as one TupleSet
// (empty when no row hashed there), as the reference's forced send on
// completion does; the reference also sends a slot early once it holds
// DefaultBufferSize rows, which changes no consumer's result.
class ShufflePOp : public PhysicalOp {
 public:
  ShufflePOp(std::string name, std::vector<std::string> cols)
      : PhysicalOp(std::move(name), "ShufflePOp"), cols_(std::move(cols)) {}

  void onReceive(const Envelope& env) override {
    const Message& m = env.getMessage();
    if (m.type == MessageType::TUPLESET) {
      const int64_t slots = static_cast<int64_t>(consumers().size());
      if (slots == 0) fail(GFPDB_EINVAL, "ShufflePOp '" + name_ + "' has no consumers");
      buffers_.resize(slots);
      TupleSetPtr in = m.tuples;
      if (!projectColumnNames_.empty()) in = in->project_exist(projectColumnNames_);
      ShuffleResult r = shuffle_rows(in, cols_, slots, ctx()->stream());
      for (int64_t i = 0; i < slots; ++i)
        buffers_[i].push_back(slice_rows(r.rows, r.offsets[i], r.offsets[i + 1] - r.offsets[i]));
    } else if (m.type == MessageType::COMPLETE) {
      if (!is_producer_complete(*this)) return;
      for (size_t i = 0; i < buffers_.size(); ++i) {
        Message out;
        out.type = MessageType::TUPLESET;
        out.tuples = buffers_[i].size() == 1 ? buffers_[i][0] : TupleSet::concatenate(buffers_[i], ctx()->stream());
        ctx()->tell(out, {consumers()[i]});
      }
      buffers_.clear();
      ctx()->notifyComplete();
    }
  }

  void clear() override { buffers_.clear(); }

 private:
  std::vector<std::string> cols_;
  std::vector<std::vector<TupleSetPtr>> buffers_;
};

// ProjectPOp (fpdb-executor/src/physical/project/ProjectPOp.cpp:48-149):
// each TupleSet leaves as its pass-through columns under their new names,
// then one column per expression (evaluated by project_kernel, compiled
// against the first TupleSet's schema, as the reference builds its projector
// on the first message). The reference buffers rows up to DefaultBufferSize
// before projecting; a projection is row-wise, so each TupleSet is projected
// as it arrives, with the same rows out.
class ProjectPOp : public PhysicalOp {
 public:
  ProjectPOp(std::string name, std::vector<ExprPtr> exprs, std::vector<std::string> expr_names,
             std::vector<std::pair<std::string, std::string>> pairs)
      : PhysicalOp(std::move(name), "ProjectPOp"), exprs_(std::move(exprs)), expr_names_(std::move(expr_names)),
        pairs_(std::move(pairs)) {}

  void onReceive(const Envelope& env) override {
    const Message& m = env.getMessage();
    if (m.type == MessageType::TUPLESET) {
      const TupleSet& in = *m.tuples;
      if (!compiled_ && !exprs_.empty()) {
        // utf8-valued expressions (a column, a SUBSTRING of one) are cut by
        // substring_column, the others evaluated by project_kernel
        utf8_.assign(exprs_.size(), Utf8Source{});
        is_utf8_.assign(exprs_.size(), false);
        for (size_t i = 0; i < exprs_.size(); ++i) {
          if (utf8_source(exprs_[i], in.fields(), &utf8_[i])) {
            is_utf8_[i] = true;
            continue;
          }
          DType t = DType::Int64;
          spec_.ops.push_back(compile_value(exprs_[i], in.fields(), spec_.prog, spec_.slots, &t));
          spec_.types.push_back(t);
          spec_.names.push_back(expr_names_[i]);
        }
        compiled_ = true;
      }
      std::vector<Field> fields;
      std::vector<ColumnPtr> cols;
      for (const auto& pr : pairs_) {
        const int ci = in.require_column(pr.first);
        fields.push_back(Field{pr.second, in.field(ci).type});
        cols.push_back(in.column(ci));
      }
      if (!exprs_.empty()) {
        for (const auto& name : spec_.slots.names) {
          const int ci = in.column_index(name);
          if (ci >= 0 && in.column(ci)->valid != nullptr)
            fail(GFPDB_EUNSUPPORTED, "ProjectPOp '" + name_ + "': an expression over the nullable column '" + name +
                                         "' (an outer join's output)");
        }
        bool any_utf8 = false;
        for (size_t i = 0; i < exprs_.size(); ++i) {
          if (!is_utf8_[i]) continue;
          any_utf8 = true;
          const int ci = in.require_column(utf8_[i].column);
          if (in.column(ci)->valid != nullptr)
            fail(GFPDB_EUNSUPPORTED, "ProjectPOp '" + name_ + "': an expression over the nullable column '" +
                                         utf8_[i].column + "' (an outer join's output)");
        }
        // utf8 outputs are sized from the exact row count
        TupleSetPtr exact = any_utf8 && !in.exact() ? in.resolve(ctx()->stream()) : nullptr;
        const TupleSet& src = exact ? *exact : in;
        TupleSetPtr e = spec_.ops.empty() ? nullptr : project_columns(spec_, src, ctx()->stream());
        int fixed_at = 0;
        for (size_t i = 0; i < exprs_.size(); ++i) {
          if (is_utf8_[i]) {
            const Utf8Source& u = utf8_[i];
            fields.push_back(Field{expr_names_[i], DType::Utf8});
            cols.push_back(substring_column(*src.column(u.column), src.num_rows(), u.sub, u.from, u.len,
                                            ctx()->stream()));
          } else {
            fields.push_back(e->field(fixed_at));
            cols.push_back(e->column(fixed_at));
            ++fixed_at;
          }
        }
        if (exact) {
          Message out;
          out.type = MessageType::TUPLESET;
          out.tuples = TupleSet::make(std::move(fields), std::move(cols), exact->num_rows());
          ctx()->tell(out);
          return;
        }
      }
      Message out;
      out.type = MessageType::TUPLESET;
      out.tuples = in.exact() ? TupleSet::make(std::move(fields), std::move(cols), in.num_rows())
                              : TupleSet::make_deferred(std::move(fields), std::move(cols), in.num_rows(),
                                                        in.rows_owner(), in.rows_dev());
      ctx()->tell(out);
    } else if (m.type == MessageType::COMPLETE) {
      if (is_producer_complete(*this)) ctx()->notifyComplete();
    }
  }

 private:
  std::vector<ExprPtr> exprs_;
  std::vector<std::string> expr_names_;
  std::vector<std::pair<std::string, std::string>> pairs_;
  ProjectSpec spec_;
  std::vector<Utf8Source> utf8_;
  std::vector<bool> is_utf8_;
  bool compiled_ = false;
};

// LimitSortPOp (fpdb-executor/src/physical/limitsort/LimitSortPOp.cpp:44-142):
// the k first rows in sort-key order of everything it receives, projected to
// projectColumnNames, sent once all producers are complete. The reference
// re-selects k after every TupleSet; the k first rows of all of them are the
// same rows, selected here once (select_k_kernel) when the input is complete.
class LimitSortPOp : public PhysicalOp {
 public:
  LimitSortPOp(std::string name, int64_t k, std::vector<SortKeySpec> keys)
      : PhysicalOp(std::move(name), "LimitSortPOp"), k_(k), keys_(std::move(keys)) {}

  void onReceive(const Envelope& env) override {
    const Message& m = env.getMessage();
    if (m.type == MessageType::TUPLESET) {
      received_.push_back(m.tuples);
    } else if (m.type == MessageType::COMPLETE) {
      if (!is_producer_complete(*this)) return;
      if (received_.empty()) {
        ctx()->notifyError("Result not produced yet");  // as the reference: no input, no result
        return;
      }
      TupleSetPtr all = received_.size() == 1 ? received_[0] : TupleSet::concatenate(received_, ctx()->stream());
      TupleSetPtr r = select_k(all, keys_, k_, ctx()->stream());
      if (!projectColumnNames_.empty()) r = r->project_exist(projectColumnNames_);
      Message out;
      out.type = MessageType::TUPLESET;
      out.tuples = r;
      ctx()->tell(out);
      ctx()->notifyComplete();
    }
  }

  void clear() override { received_.clear(); }

 private:
  int64_t k_;
  std::vector<SortKeySpec> keys_;
  std::vector<TupleSetPtr> received_;
};

// Parses delimited text into a TupleSet: the CSV branch of the reference's
// file scans (FileScanAbstractPOp::readAndSendTuples reading through
// CSVReader::read, fpdb-tuple/src/csv/CSVReader.cpp:15-21), reading the text
// from an input table whose first column is a single utf8 value (the file's
// bytes) instead of a file. Only the projected fields are materialised.
class CsvScanPOp : public PhysicalOp {
 public:
  CsvScanPOp(std::string name, std::string table, std::vector<CsvField> fields, std::vector<int> emit, char delim,
             bool header)
      : PhysicalOp(std::move(name), "CsvScanPOp"), table_(std::move(table)), fields_(std::move(fields)),
        emit_(std::move(emit)), delim_(delim), header_(header) {}

  void setExecution(Execution* e) { exec_ = e; }

  void onReceive(const Envelope& env) override {
    const Message& m = env.getMessage();
    if (m.type != MessageType::START) return;
    const InputTable& in = exec_->input(table_);
    TupleSetPtr ts = in.device ? in.device : import_tupleset(in.schema, in.array, ctx()->stream());
    ts = resolved(ts, ctx()->stream());
    if (ts->num_columns() < 1 || ts->field(0).type != DType::Utf8 || ts->num_rows() != 1)
      fail(GFPDB_EINVAL, "CsvScanPOp input '" + table_ + "' must hold the text as one utf8 value");
    const auto& c = ts->column(0);
    int32_t off[2];
    GF_CUDA(cudaMemcpyAsync(off, c->offsets, sizeof(off), cudaMemcpyDeviceToHost, ctx()->stream()));
    sync(ctx()->stream());
    const char* text = static_cast<const char*>(c->data) + off[0];
    Message out;
    out.type = MessageType::TUPLESET;
    out.tuples = csv_parse(text, off[1] - off[0], delim_, header_, fields_, emit_, ctx()->stream());
    ctx()->tell(out);
    ctx()->notifyComplete();
  }

 private:
  Execution* exec_ = nullptr;
  std::string table_;
  std::vector<CsvField> fields_;
  std::vector<int> emit_;
  char delim_;
  bool header_;
};

// The bytes of an input table holding one value (a file's contents), in
// host memory: read in place from a host array, copied from a device one.
std::vector<uint8_t> input_bytes(const InputTable& in, const std::string& table, cudaStream_t s) {
  if (in.array != nullptr && (in.array->device_type == ARROW_DEVICE_CPU || in.array->device_type == ARROW_DEVICE_CUDA_HOST)) {
    const ArrowArray& a = in.array->array;
    if (a.n_children < 1 || a.children[0]->n_buffers != 3 || a.length != 1)
      fail(GFPDB_EINVAL, "input '" + table + "' must hold the file as one utf8 value");
    const ArrowArray* c = a.children[0];
    const int32_t* offs = static_cast<const int32_t*>(c->buffers[1]) + c->offset + a.offset;
    const uint8_t* data = static_cast<const uint8_t*>(c->buffers[2]);
    return std::vector<uint8_t>(data + offs[0], data + offs[1]);
  }
  TupleSetPtr ts = in.device ? in.device : import_tupleset(in.schema, in.array, s);
  ts = resolved(ts, s);
  if (ts->num_columns() < 1 || ts->field(0).type != DType::Utf8 || ts->num_rows() != 1)
    fail(GFPDB_EINVAL, "input '" + table + "' must hold the file as one utf8 value");
  const auto& c = ts->column(0);
  int32_t off[2];
  GF_CUDA(cudaMemcpyAsync(off, c->offsets, sizeof(off), cudaMemcpyDeviceToHost, s));
  sync(s);
  std::vector<uint8_t> bytes(static_cast<size_t>(off[1] - off[0]));
  if (!bytes.empty())
    GF_CUDA(cudaMemcpyAsync(bytes.data(), static_cast<const uint8_t*>(c->data) + off[0], bytes.size(),
                            cudaMemcpyDeviceToHost, s));
  sync(s);
  return bytes;
}

// ParquetScanPOp: the Parquet file held by an input table decoded into its
// columns (ParquetReader::read / readRange,
// fpdb-tuple/src/parquet/ParquetReader.cpp:12-120, as FileScanAbstractPOp
// reads a Parquet object, FileScanAbstractPOp.cpp:73-130).
class ParquetScanPOp : public PhysicalOp {
 public:
  ParquetScanPOp(std::string name, std::string table, std::vector<std::string> columns, int64_t start, int64_t end)
      : PhysicalOp(std::move(name), "ParquetScanPOp"), table_(std::move(table)), columns_(std::move(columns)),
        start_(start), end_(end) {}

  void setExecution(Execution* e) { exec_ = e; }

  void onReceive(const Envelope& env) override {
    if (env.getMessage().type != MessageType::START) return;
    const std::vector<uint8_t> bytes = input_bytes(exec_->input(table_), table_, ctx()->stream());
    Message out;
    out.type = MessageType::TUPLESET;
    out.tuples = parquet_read(bytes.data(), static_cast<int64_t>(bytes.size()), columns_, start_, end_,
                              ctx()->stream());
    ctx()->tell(out);
    ctx()->notifyComplete();
  }

 private:
  Execution* exec_ = nullptr;
  std::string table_;
  std::vector<std::string> columns_;
  int64_t start_, end_;
};

// FileScanPOp over a local file (FileScanAbstractPOp::readAndSendTuples with
// LocalFileScanKernel::scan, fpdb-executor/src/physical/file/FileScanAbstractPOp.cpp:73-130,
// LocalFileScanKernel.cpp:38-91): the file is read from the file system,
// then parsed on the device as CSV (csv_parse) or Parquet (parquet_read).
class FileScanPOp : public PhysicalOp {
 public:
  FileScanPOp(std::string name, std::string path, bool parquet, std::vector<std::string> columns, int64_t start,
              int64_t end, std::vector<CsvField> fields, std::vector<int> emit, char delim, bool header)
      : PhysicalOp(std::move(name), "FileScanPOp"), path_(std::move(path)), parquet_(parquet),
        columns_(std::move(columns)), start_(start), end_(end), fields_(std::move(fields)), emit_(std::move(emit)),
        delim_(delim), header_(header) {}

  void onReceive(const Envelope& env) override {
    if (env.getMessage().type != MessageType::START) return;
    const std::vector<uint8_t> bytes = read_local_file(path_);
    Message out;
    out.type = MessageType::TUPLESET;
    if (parquet_) {
      out.tuples = parquet_read(bytes.data(), static_cast<int64_t>(bytes.size()), columns_, start_, end_,
                                ctx()->stream());
    } else {
      auto text = make_buffer(static_cast<int64_t>(bytes.size()) > 0 ? static_cast<int64_t>(bytes.size()) : 1,
                              ctx()->stream());
      copy_h2d(text->data(), bytes.data(), static_cast<int64_t>(bytes.size()), ctx()->stream());
      out.tuples = csv_parse(text->as<char>(), static_cast<int64_t>(bytes.size()), delim_, header_, fields_, emit_,
                             ctx()->stream());
      sync(ctx()->stream());  // `bytes` and `text` go when this returns
    }
    ctx()->tell(out);
    ctx()->notifyComplete();
  }

 private:
  std::string path_;
  bool parquet_;
  std::vector<std::string> columns_;
  int64_t start_, end_;
  std::vector<CsvField> fields_;
  std::vector<int> emit_;
  char delim_;
  bool header_;
};

// CollatePOp (fpdb-executor/src/physical/collate/CollatePOp.cpp:67-150):
// concatenates everything it receives into the query result.
class CollatePOp : public PhysicalOp {
 public:
  explicit CollatePOp(std::string name) : PhysicalOp(std::move(name), "CollatePOp") {}

  void onReceive(const Envelope& env) override {
    const Message& m = env.getMessage();
    if (m.type == MessageType::TUPLESET) {
      received_.push_back(m.tuples);
    } else if (m.type == MessageType::COMPLETE) {
      if (!is_producer_complete(*this)) return;
      if (!received_.empty()) result_ = TupleSet::concatenate(received_, ctx()->stream());
      ctx()->notifyComplete();
    }
  }

  TupleSetPtr tuples() const { return result_; }

 private:
  std::vector<TupleSetPtr> received_;
  TupleSetPtr result_;
};

AggFn agg_fn(const std::string& f) {
  if (f == "SUM" || f == "sum" || f == "Sum") return AGG_SUM;
  if (f == "COUNT" || f == "count" || f == "Count") return AGG_COUNT;
  if (f == "MIN" || f == "min" || f == "Min") return AGG_MIN;
  if (f == "MAX" || f == "max" || f == "Max") return AGG_MAX;
  if (f == "AVG" || f == "avg" || f == "Avg") return AGG_AVG;
  if (f == "AVG_REDUCE" || f == "AvgReduce") return AGG_AVG_REDUCE;
  fail(GFPDB_EUNSUPPORTED, "aggregate function '" + f + "'");
}

}  // namespace

std::vector<uint8_t> read_local_file(const std::string& path) {
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (f == nullptr) fail(GFPDB_EINVAL, "cannot open '" + path + "'");
  std::vector<uint8_t> bytes;
  uint8_t buf[1 << 16];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) bytes.insert(bytes.end(), buf, buf + got);
  const bool bad = std::ferror(f) != 0;
  std::fclose(f);
  if (bad) fail(GFPDB_EINVAL, "cannot read '" + path + "'");
  return bytes;
}

std::vector<GroupAggregate> parse_aggregates(const json::Value& list) {
  std::vector<GroupAggregate> aggs;
  for (auto& a : list.array()) {
    GroupAggregate g;
    g.fn = agg_fn(a.at("function").str());
    g.name = a.at("name").str();
    if (a.contains("expr") && a.at("expr").kind != json::Value::Null) g.expr = parse_expr(a.at("expr"));
    else if (g.fn == AGG_COUNT) g.fn = AGG_COUNT_STAR;
    else if (g.fn != AGG_AVG_REDUCE) fail(GFPDB_EINVAL, "aggregate '" + g.name + "' needs an expr");
    if (g.fn == AGG_AVG_REDUCE && g.expr) fail(GFPDB_EINVAL, "AVG_REDUCE '" + g.name + "' takes no expression");
    aggs.push_back(g);
  }
  return aggs;
}

// --------------------------------------------------------------- Execution

void Execution::add(std::unique_ptr<PhysicalOp> op) {
  if (by_name_.count(op->name())) fail(GFPDB_EINVAL, "duplicate operator name '" + op->name() + "'");
  op->setContext(std::make_unique<POpContext>(this, op.get()));
  by_name_[op->name()] = op.get();
  ops_.push_back(std::move(op));
}

PhysicalOp* Execution::op(const std::string& name) {
  auto it = by_name_.find(name);
  if (it == by_name_.end()) fail(GFPDB_EINVAL, "unknown operator '" + name + "'");
  return it->second;
}

void Execution::connect() {
  for (auto& o : ops_)
    for (auto& c : o->consumers()) {
      PhysicalOp* dst = op(c);
      if (std::find(dst->producers().begin(), dst->producers().end(), o->name()) == dst->producers().end())
        dst->producers().push_back(o->name());
    }
  for (auto& o : ops_) {
    for (auto& p : o->producers()) o->directory().add(p, POpRelationshipType::Producer);
    for (auto& c : o->consumers()) o->directory().add(c, POpRelationshipType::Consumer);
  }
  stats_.num_ops = static_cast<int64_t>(ops_.size());
}

const InputTable& Execution::input(const std::string& name) const {
  auto it = inputs_.find(name);
  if (it == inputs_.end()) fail(GFPDB_EINVAL, "plan scans table '" + name + "' but no such table was passed");
  return it->second;
}

void Execution::post(const std::string& to, Message msg) { mailbox_.emplace_back(to, std::move(msg)); }

namespace {

// This thread's secondary streams and events for the current device, created
// on first use and kept (creating them is not free, and a graph capture must
// not be the first to need one).
struct StreamPool {
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;
};

StreamPool& stream_pool() {
  thread_local std::map<int, StreamPool> pools;
  int dev = 0;
  GF_CUDA(cudaGetDevice(&dev));
  return pools[dev];
}

cudaStream_t pooled_stream(size_t i) {
  StreamPool& p = stream_pool();
  while (p.streams.size() <= i) {
    cudaStream_t s = nullptr;
    GF_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    p.streams.push_back(s);
  }
  return p.streams[i];
}

cudaEvent_t pooled_event(size_t i) {
  StreamPool& p = stream_pool();
  while (p.events.size() <= i) {
    cudaEvent_t e = nullptr;
    GF_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    p.events.push_back(e);
  }
  return p.events[i];
}

}  // namespace

Execution::~Execution() = default;

// Streams by position in the plan: an operator continues its first producer's
// stream unless another consumer of that producer already did; roots and
// branches take the next stream in turn.
void Execution::assignStreams() {
  streams_.assign(1, stream_);
  op_stream_.clear();
  if (n_streams_ <= 1) {
    for (auto& o : ops_) op_stream_[o.get()] = 0;
    return;
  }
  for (int i = 1; i < n_streams_; ++i) streams_.push_back(pooled_stream(static_cast<size_t>(i - 1)));
  // topological order over producers
  std::map<std::string, int> indeg;
  for (auto& o : ops_) indeg[o->name()] = static_cast<int>(o->producers().size());
  std::deque<PhysicalOp*> ready;
  for (auto& o : ops_)
    if (o->producers().empty()) ready.push_back(o.get());
  std::set<const PhysicalOp*> continued;  // producers whose stream a consumer took
  int next = 0;
  auto fresh = [&]() { return next++ % n_streams_; };
  std::set<std::string> seen;
  while (!ready.empty()) {
    PhysicalOp* o = ready.front();
    ready.pop_front();
    if (!seen.insert(o->name()).second) continue;
    int st = -1;
    for (auto& pn : o->producers()) {
      const PhysicalOp* p = op(pn);
      // filter builds along a chain of BloomFilterCreatePOps run side by side
      if (p->getTypeString() == "BloomFilterCreatePOp" && o->getTypeString() == "BloomFilterCreatePOp") continue;
      if (!continued.count(p)) {
        continued.insert(p);
        st = op_stream_[p];
        break;
      }
    }
    op_stream_[o] = st >= 0 ? st : fresh();
    for (auto& cn : o->consumers())
      if (--indeg[cn] == 0) ready.push_back(op(cn));
  }
  for (auto& o : ops_)
    if (!op_stream_.count(o.get())) op_stream_[o.get()] = 0;  // not reached (cycles): the caller's stream
}

cudaStream_t Execution::streamOf(const PhysicalOp* op) const {
  auto it = op_stream_.find(op);
  return it == op_stream_.end() || streams_.empty() ? stream_ : streams_[it->second];
}

cudaStream_t Execution::sideStreamOf(const PhysicalOp* op, int k) const {
  if (streams_.size() <= 1) return streamOf(op);
  auto it = op_stream_.find(op);
  const int own = it == op_stream_.end() ? 0 : it->second;
  return streams_[static_cast<size_t>(own + 1 + k) % streams_.size()];
}

void Execution::streamWait(cudaStream_t waiter, cudaStream_t on) {
  if (waiter == on) return;
  cudaEvent_t e = pooled_event(events_used_++);
  GF_CUDA(cudaEventRecord(e, on));
  GF_CUDA(cudaStreamWaitEvent(waiter, e, 0));
}

void Execution::stamp(Message& msg, const PhysicalOp* sender) {
  if (streams_.size() <= 1) return;
  // A COMPLETE carries no device dependency: every TUPLESET and BLOOM_FILTER
  // before it was waited for on arrival, and ordering work after the
  // sender's own later kernels would only serialise independent operators
  // (a chain of BloomFilterCreatePOps, each forwarding its input, would
  // build its filters one after another).
  if (msg.type == MessageType::COMPLETE) return;
  auto it = op_stream_.find(sender);
  msg.stream = it == op_stream_.end() ? 0 : it->second;
  msg.ready = pooled_event(events_used_++);
  GF_CUDA(cudaEventRecord(msg.ready, streams_[msg.stream]));
  if (msg.tuples) retained_tuples_.push_back(msg.tuples);
  if (msg.bloom) retained_blooms_.push_back(msg.bloom);
}

void Execution::markComplete(const std::string&) {}

void Execution::error(const std::string& from, const std::string& msg) {
  if (error_.empty()) error_ = "operator '" + from + "': " + msg;
}

TupleSetPtr Execution::execute() {
  const uint64_t launches0 = g_kernel_launches.load();
  const CopyCounters c0 = copy_counters();
  assignStreams();
  events_used_ = 0;
  // Fork: every secondary stream starts after the work already on the
  // caller's stream (and, under capture, joins the capture).
  if (streams_.size() > 1) {
    cudaEvent_t fork = pooled_event(events_used_++);
    GF_CUDA(cudaEventRecord(fork, stream_));
    for (size_t i = 1; i < streams_.size(); ++i) GF_CUDA(cudaStreamWaitEvent(streams_[i], fork, 0));
  }
  // Join: the caller's stream waits for every secondary stream, on every
  // exit path (a capture cannot end with unjoined streams).
  struct JoinGuard {
    Execution* e;
    ~JoinGuard() {
      for (size_t i = 1; i < e->streams_.size(); ++i) {
        cudaEvent_t j = nullptr;
        try {
          j = pooled_event(e->events_used_++);
        } catch (...) {
          return;
        }
        (void)cudaEventRecord(j, e->streams_[i]);
        (void)cudaStreamWaitEvent(e->stream_, j, 0);
      }
    }
  };
  std::optional<JoinGuard> join_guard;
  join_guard.emplace(JoinGuard{this});
  for (auto& o : ops_) {
    Message start;
    start.type = MessageType::START;
    start.sender = "root";
    post(o->name(), start);
  }
  int32_t code = GFPDB_EINVAL;
  clear_deferred_checks();
  set_deferred_mode(deferred_);
  struct ModeGuard {
    ~ModeGuard() { set_deferred_mode(false); }
  } mode_guard;
  while (!mailbox_.empty() && error_.empty()) {
    auto [to, msg] = std::move(mailbox_.front());
    mailbox_.pop_front();
    PhysicalOp* dst = op(to);
    if (dst->ctx()->isComplete()) continue;
    ++stats_.messages;
    if (msg.ready != nullptr) {
      const int ds = op_stream_.count(dst) ? op_stream_[dst] : 0;
      if (ds != msg.stream) GF_CUDA(cudaStreamWaitEvent(streams_[ds], msg.ready, 0));
    }
    if (msg.type == MessageType::COMPLETE) dst->directory().setComplete(msg.sender);
    try {
      // Nullable columns (outer-join outputs) go only where they are passed
      // through unchanged: the collate, and a projection's renamed columns
      // (ProjectPOp checks its expressions); every other operator's kernels
      // read values, not nulls, and refuse them.
      if (msg.type == MessageType::TUPLESET && msg.tuples && has_nulls(*msg.tuples)) {
        const std::string t = dst->getTypeString();
        if (t != "CollatePOp" && t != "ProjectPOp")
          fail(GFPDB_EUNSUPPORTED, t + " '" + dst->name() + "' does not take nullable columns (column '" +
                                       first_nullable_column(*msg.tuples) + "', an outer join's output)");
      }
      dst->onReceive(Envelope{msg});
    } catch (const Error& e) {
      code = e.code();
      dst->ctx()->notifyError(e.what());
    } catch (const std::exception& e) {
      dst->ctx()->notifyError(e.what());
    }
  }
  set_deferred_mode(false);
  join_guard.reset();  // join the streams before anything waits on the caller's stream
  if (!error_.empty()) {
    clear_deferred_checks();
    // Operators free their buffers on their own streams when the execution
    // goes away; on this path some were not ordered after the work that
    // uses them, so let everything issued finish first (nothing is freed
    // under capture: the graph's memory is an arena).
    if (!capturing_) (void)cudaStreamSynchronize(stream_);
    fail(code, error_);
  }
  if (capturing_) {
    // Under graph capture nothing may wait: the checks run after each replay.
    captured_checks_ = take_deferred_checks();
  } else if (deferred_) {
    // One synchronization for the whole plan: device errors of every
    // operator, and whether every deferred output fit its capacity.
    sync(stream_);
    if (!run_deferred_checks(stream_)) throw NeedsExactSizes();
  }
  std::string incomplete;
  CollatePOp* collate = nullptr;
  for (auto& o : ops_) {
    if (!o->ctx()->isComplete()) incomplete += (incomplete.empty() ? "" : ", ") + o->name();
    if (auto* c = dynamic_cast<CollatePOp*>(o.get())) collate = c;
  }
  if (!incomplete.empty()) fail(GFPDB_EINVAL, "plan finished with incomplete operators: " + incomplete);
  if (collate == nullptr) fail(GFPDB_EINVAL, "plan has no CollatePOp");
  stats_.kernel_launches = static_cast<int64_t>(g_kernel_launches.load() - launches0);
  stats_.h2d_bytes = copy_counters().h2d - c0.h2d + copy_counters().in_place - c0.in_place;
  stats_.d2h_bytes = copy_counters().d2h - c0.d2h;
  TupleSetPtr r = collate->tuples();
  if (!r) fail(GFPDB_EINVAL, "CollatePOp received no TupleSet");
  return r;
}

// ------------------------------------------------------------ plan parsing

namespace {

std::unique_ptr<PhysicalOp> make_op(const json::Value& o, Execution* exec) {
  const std::string type = o.at("type").str();
  const std::string name = o.at("name").str();
  std::unique_ptr<PhysicalOp> op;
  if (type == "TableScanPOp") {
    auto s = std::make_unique<TableScanPOp>(name, o.at("table").str(), o.str_list("columns"), o.get_int("chunkRows", 0),
                                            o.str_list("inPlaceColumns"));
    s->setExecution(exec);
    op = std::move(s);
  } else if (type == "FilterPOp") {
    op = std::make_unique<FilterPOp>(name, parse_expr(o.at("predicate")));
  } else if (type == "BloomFilterCreatePOp") {
    // one filter, or several ("filters": [{"origin", "bloomFilterColumn",
    // "bitsPerKey", "numHashes", "bloomFilterUsePOps"}], fused creators)
    std::vector<CreatedFilter> filters;
    auto one = [&](const json::Value& f, const std::string& origin) {
      CreatedFilter c;
      c.origin = origin;
      c.column = f.at("bloomFilterColumn").str();
      c.bits = static_cast<int>(f.get_int("bitsPerKey", 10));
      c.hashes = static_cast<int>(f.get_int("numHashes", 3));
      c.uses = f.str_list("bloomFilterUsePOps");
      filters.push_back(std::move(c));
    };
    if (o.contains("filters"))
      for (auto& f : o.at("filters").array()) one(f, f.get_str("origin", name));
    else
      one(o, name);
    op = std::make_unique<BloomFilterCreatePOp>(name, std::move(filters),
                                                o.contains("dataConsumers")
                                                    ? std::optional<std::vector<std::string>>(o.str_list("dataConsumers"))
                                                    : std::nullopt);
  } else if (type == "BloomFilterUsePOp") {
    std::vector<std::string> cols = o.contains("bloomFilterColumns") ? o.str_list("bloomFilterColumns")
                                                                     : std::vector<std::string>{o.at("bloomFilterColumn").str()};
    std::vector<std::string> creators = o.str_list("creators");
    if (!creators.empty() && creators.size() != cols.size())
      fail(GFPDB_EINVAL, "BloomFilterUsePOp '" + name + "': one creator per filter column");
    op = std::make_unique<BloomFilterUsePOp>(name, cols, creators);
  } else if (type == "HashJoinArrowPOp") {
    const JoinKind kind = join_kind_from_name(o.get_str("joinType", "INNER"));
    // one key column per side ("buildKey" / "probeKey") or lists of them
    // ("buildKeys" / "probeKeys", HashJoinPredicate.h:25-26)
    std::vector<std::string> bk = o.contains("buildKeys") ? o.str_list("buildKeys")
                                                          : std::vector<std::string>{o.at("buildKey").str()};
    std::vector<std::string> pk = o.contains("probeKeys") ? o.str_list("probeKeys")
                                                          : std::vector<std::string>{o.at("probeKey").str()};
    if (kind != JoinKind::Inner && bk.size() != 1)
      fail(GFPDB_EUNSUPPORTED, "HashJoinArrowPOp '" + name + "': outer and semi joins take one key column per side");
    op = std::make_unique<HashJoinArrowPOp>(name, o.str_list("buildProducers"), o.str_list("probeProducers"),
                                            std::move(bk), std::move(pk), o.get_num("loadFactor", 0.5), kind,
                                            parse_build_filters(o));
  } else if (type == "HashJoinChainPOp") {
    std::vector<ChainJoinSpec> joins;
    for (auto& j : o.at("joins").array()) {
      std::string jt = j.get_str("joinType", "INNER");
      if (jt != "INNER") fail(GFPDB_EUNSUPPORTED, "join type '" + jt + "' (only INNER runs on the GPU path)");
      ChainJoinSpec c;
      c.name = j.get_str("name", name);
      c.build_producers = j.str_list("buildProducers");
      c.build_key = j.at("buildKey").str();
      c.probe_key = j.at("probeKey").str();
      c.load_factor = j.get_num("loadFactor", 0.5);
      c.proj = j.str_list("projectColumnNames");
      c.filters = parse_build_filters(j);
      joins.push_back(std::move(c));
    }
    op = std::make_unique<HashJoinChainPOp>(name, std::move(joins));
  } else if (type == "CsvScanPOp" || (type == "FileScanPOp" && o.get_str("format", "csv") == "csv")) {
    std::vector<CsvField> fields;
    for (auto& f : o.at("fields").array()) {
      CsvField cf;
      cf.name = f.at("name").str();
      const std::string ty = f.at("type").str();
      if (ty.rfind("decimal", 0) == 0) {
        const auto comma = ty.find(',');
        if (comma == std::string::npos) fail(GFPDB_EINVAL, "decimal field types are written decimal(p,s)");
        cf.type = DType::Int64;
        cf.decimal = true;
        cf.scale = std::atoi(ty.c_str() + comma + 1);
        if (cf.scale < 0 || cf.scale > 9) fail(GFPDB_EINVAL, "decimal scale must be in [0, 9]");
      } else {
        cf.type = dtype_from_name(ty);
      }
      fields.push_back(cf);
    }
    std::vector<int> emit;
    if (o.contains("columns")) {
      for (auto& cn : o.str_list("columns")) {
        int found = -1;
        for (size_t i = 0; i < fields.size(); ++i)
          if (fields[i].name == cn) found = static_cast<int>(i);
        if (found < 0) fail(GFPDB_EINVAL, type + " '" + name + "': column '" + cn + "' is not a field");
        emit.push_back(found);
      }
    } else {
      for (size_t i = 0; i < fields.size(); ++i) emit.push_back(static_cast<int>(i));
    }
    const std::string delim = o.get_str("delimiter", ",");
    if (delim.size() != 1) fail(GFPDB_EINVAL, type + " delimiter must be one byte");
    if (type == "FileScanPOp") {
      op = std::make_unique<FileScanPOp>(name, o.at("path").str(), false, std::vector<std::string>{}, 0, -1,
                                         std::move(fields), std::move(emit), delim[0], o.get_bool("header", false));
    } else {
      auto cs = std::make_unique<CsvScanPOp>(name, o.at("table").str(), std::move(fields), std::move(emit), delim[0],
                                             o.get_bool("header", false));
      cs->setExecution(exec);
      op = std::move(cs);
    }
  } else if (type == "FileScanPOp") {
    const std::string fmt = o.get_str("format", "csv");
    if (fmt != "parquet") fail(GFPDB_EUNSUPPORTED, "FileScanPOp '" + name + "': format '" + fmt + "' (csv or parquet)");
    op = std::make_unique<FileScanPOp>(name, o.at("path").str(), true, o.str_list("columns"),
                                       o.get_int("startPos", 0), o.get_int("finishPos", -1), std::vector<CsvField>{},
                                       std::vector<int>{}, ',', false);
  } else if (type == "ParquetScanPOp") {
    auto ps = std::make_unique<ParquetScanPOp>(name, o.at("table").str(), o.str_list("columns"),
                                               o.get_int("startPos", 0), o.get_int("finishPos", -1));
    ps->setExecution(exec);
    op = std::move(ps);
  } else if (type == "GroupPOp" || type == "AggregatePOp") {
    std::vector<GroupAggregate> aggs = parse_aggregates(o.at("aggregates"));
    if (type == "AggregatePOp") {
      // AggregatePOp (fpdb-executor/src/physical/aggregate/AggregatePOp.cpp:57-153):
      // the non-grouped aggregate, run as a group-by with one implicit group.
      op = std::make_unique<GroupPOp>(name, std::vector<std::string>{}, aggs, 1, "AggregatePOp");
    } else {
      op = std::make_unique<GroupPOp>(name, o.str_list("groupColumnNames"), aggs, o.get_int("groupsHint", 0));
    }
  } else if (type == "ProjectPOp") {
    std::vector<ExprPtr> exprs;
    std::vector<std::string> expr_names;
    if (o.contains("exprs"))
      for (auto& e : o.at("exprs").array()) {
        exprs.push_back(parse_expr(e.at("expr")));
        expr_names.push_back(e.at("name").str());
      }
    std::vector<std::pair<std::string, std::string>> pairs;
    if (o.contains("projectColumnNamePairs"))
      for (auto& pr : o.at("projectColumnNamePairs").array()) {
        if (pr.kind != json::Value::Array || pr.a.size() != 2)
          fail(GFPDB_EINVAL, "ProjectPOp '" + name + "': projectColumnNamePairs holds [input, output] pairs");
        pairs.emplace_back(pr.a[0].str(), pr.a[1].str());
      }
    if (exprs.size() > static_cast<size_t>(kMaxProjOut))
      fail(GFPDB_EUNSUPPORTED, "ProjectPOp '" + name + "': more than 16 expressions");
    op = std::make_unique<ProjectPOp>(name, std::move(exprs), std::move(expr_names), std::move(pairs));
  } else if (type == "LimitSortPOp") {
    std::vector<SortKeySpec> keys;
    for (auto& k : o.at("sortKeys").array()) {
      const std::string order = k.get_str("order", "ASC");
      if (order != "ASC" && order != "DESC")
        fail(GFPDB_EINVAL, "LimitSortPOp '" + name + "': sort order is ASC or DESC");
      keys.push_back(SortKeySpec{k.at("name").str(), order == "DESC"});
    }
    const int64_t k = o.get_int("k", -1);
    if (keys.empty() || keys.size() > static_cast<size_t>(kMaxSortKeys))
      fail(GFPDB_EUNSUPPORTED, "LimitSortPOp '" + name + "': 1 to 4 sort keys");
    if (k < 0 || k > 1024) fail(GFPDB_EUNSUPPORTED, "LimitSortPOp '" + name + "': k must be in [0, 1024]");
    op = std::make_unique<LimitSortPOp>(name, k, std::move(keys));
  } else if (type == "ShufflePOp") {
    std::vector<std::string> cols = o.str_list("shuffleColumnNames");
    if (cols.empty() || cols.size() > static_cast<size_t>(kMaxKeyColumns))
      fail(GFPDB_EINVAL, "ShufflePOp '" + name + "' shuffles on 1 to 8 columns");
    if (!o.contains("consumers") || o.at("consumers").array().empty())
      fail(GFPDB_EINVAL, "ShufflePOp '" + name + "' needs consumers (one slot each)");
    if (static_cast<int64_t>(o.at("consumers").array().size()) > kShuffleMaxSlots)
      fail(GFPDB_EINVAL, "ShufflePOp '" + name + "' has more consumers than shuffle slots");
    op = std::make_unique<ShufflePOp>(name, std::move(cols));
  } else if (type == "CollatePOp") {
    op = std::make_unique<CollatePOp>(name);
  } else {
    fail(GFPDB_EUNSUPPORTED, "operator type '" + type + "'");
  }
  op->consumers() = o.str_list("consumers");
  op->setProjectColumnNames(o.str_list("projectColumnNames"));
  return op;
}

}  // namespace

namespace {

json::Value jstr(const std::string& s) {
  json::Value v;
  v.kind = json::Value::String;
  v.s = s;
  return v;
}

json::Value jlist(const std::vector<std::string>& xs) {
  json::Value v;
  v.kind = json::Value::Array;
  for (auto& x : xs) v.a.push_back(jstr(x));
  return v;
}

void jset(json::Value& o, const std::string& key, json::Value v) {
  for (auto& kv : o.o)
    if (kv.first == key) {
      kv.second = std::move(v);
      return;
    }
  o.o.emplace_back(key, std::move(v));
}

json::Value* jfind(json::Value& o, const std::string& key) {
  for (auto& kv : o.o)
    if (kv.first == key) return &kv.second;
  return nullptr;
}

// Rewrites the operator names listed in o[key] in place: map(name, out)
// appends what a name becomes (nothing: it is dropped) and returns true when
// it changes, and only the first occurrence of each name is kept. A list
// whose names are all strings, none of them changed and none repeated, is
// already what the rewrite would make, and is left as it is.
template <class Map>
void rewrite_names(json::Value& o, const char* key, const Map& map) {
  json::Value* l = jfind(o, key);
  if (l == nullptr) return;
  bool rebuild = l->kind != json::Value::Array;  // str_list below reports it
  std::vector<std::string> ys;
  for (size_t i = 0; !rebuild && i < l->a.size(); ++i) {
    const json::Value& e = l->a[i];
    if (e.kind != json::Value::String) {
      rebuild = true;
      break;
    }
    ys.clear();
    if (map(e.s, ys)) rebuild = true;
    for (size_t k = 0; k < i && !rebuild; ++k) rebuild = l->a[k].s == e.s;
  }
  if (!rebuild) return;
  std::vector<std::string> nv;
  for (const auto& x : o.str_list(key)) {
    ys.clear();
    if (!map(x, ys)) ys.push_back(x);
    for (auto& y : ys)
      if (std::find(nv.begin(), nv.end(), y) == nv.end()) nv.push_back(y);
  }
  *l = jlist(nv);
}

}  // namespace

// Pipeline fusion: a chain of BloomFilterUsePOps in which each one's only
// consumer is the next, and the next's only data producer is the previous,
// becomes one BloomFilterUsePOp carrying every (column, creator) probe, so
// the fact table is scanned once instead of once per filter. The fused
// operator keeps the last one's name, so every reference to the chain's end
// stays valid. Results are unchanged: a row survives the fused pass exactly
// when it survives every filter of the chain.
void fuse_bloom_chains(std::vector<json::Value>& ops) {
  for (;;) {
    std::map<std::string, std::vector<std::string>> producers, creators;
    for (auto& o : ops) {
      for (auto& c : o.str_list("consumers")) producers[c].push_back(o.at("name").str());
      if (o.at("type").str() == "BloomFilterCreatePOp")
        for (auto& u : o.str_list("bloomFilterUsePOps")) creators[u].push_back(o.at("name").str());
    }
    auto creators_of = [&](const json::Value& u) {
      auto c = u.str_list("creators");
      return c.empty() ? creators[u.at("name").str()] : c;
    };
    auto columns_of = [&](const json::Value& u) {
      return u.contains("bloomFilterColumns") ? u.str_list("bloomFilterColumns")
                                              : std::vector<std::string>{u.at("bloomFilterColumn").str()};
    };
    int first = -1, second = -1;
    for (size_t i = 0; i < ops.size() && first < 0; ++i) {
      if (ops[i].at("type").str() != "BloomFilterUsePOp") continue;
      auto cons = ops[i].str_list("consumers");
      if (cons.size() != 1) continue;
      for (size_t j = 0; j < ops.size(); ++j) {
        if (j == i || ops[j].at("type").str() != "BloomFilterUsePOp" || ops[j].at("name").str() != cons[0]) continue;
        // the next one's data producers: its producers other than its filters' creators
        std::vector<std::string> data;
        const auto cj = creators_of(ops[j]);
        for (auto& p : producers[cons[0]])
          if (std::find(cj.begin(), cj.end(), p) == cj.end()) data.push_back(p);
        if (data != std::vector<std::string>{ops[i].at("name").str()}) break;
        if (creators_of(ops[i]).size() != columns_of(ops[i]).size()) break;
        if (creators_of(ops[j]).size() != columns_of(ops[j]).size()) break;
        first = static_cast<int>(i);
        second = static_cast<int>(j);
        break;
      }
    }
    if (first < 0) break;
    const std::string u1 = ops[first].at("name").str(), u2 = ops[second].at("name").str();
    auto cols = columns_of(ops[first]);
    auto c2 = columns_of(ops[second]);
    cols.insert(cols.end(), c2.begin(), c2.end());
    auto crs = creators_of(ops[first]);
    auto r2 = creators_of(ops[second]);
    crs.insert(crs.end(), r2.begin(), r2.end());
    jset(ops[second], "bloomFilterColumns", jlist(cols));
    jset(ops[second], "creators", jlist(crs));
    auto to_u2 = [&](const std::string& x, std::vector<std::string>& out) {
      if (x != u1) return false;
      out.push_back(u2);
      return true;
    };
    for (auto& o : ops)
      for (const char* key : {"consumers", "bloomFilterUsePOps", "buildProducers", "probeProducers", "dataConsumers"})
        rewrite_names(o, key, to_u2);
    ops.erase(ops.begin() + first);
  }
}

// Pipeline fusion: a BloomFilterUsePOp whose only consumer is an inner
// HashJoinArrowPOp on one key column, which takes it as its only build
// producer, and whose filters are all on that key, is folded into the join: its data
// producers feed the join's build side directly, its filters' creators send
// them to the join ("buildFilters"), and the join build leaves out the rows
// a filter rejects (join_build_table) instead of a selection pass copying
// the rows that pass. Results are unchanged: an inner join emits a build row
// only with a probe row that finds it, and the rows the selection would have
// dropped are never found. Each creator's ordinary consumers are written out
// ("dataConsumers") first, since the join may also take the creator's rows.
void fuse_build_filters(std::vector<json::Value>& ops) {
  auto index_of = [&](const std::string& name) {
    for (size_t i = 0; i < ops.size(); ++i)
      if (ops[i].at("name").str() == name) return static_cast<int>(i);
    return -1;
  };
  for (;;) {
    std::map<std::string, std::vector<std::string>> producers, creators;
    for (auto& o : ops) {
      for (auto& c : o.str_list("consumers")) producers[c].push_back(o.at("name").str());
      if (o.at("type").str() == "BloomFilterCreatePOp")
        for (auto& u : o.str_list("bloomFilterUsePOps")) creators[u].push_back(o.at("name").str());
    }
    int use = -1, join = -1;
    std::vector<std::string> cols, crs;
    for (size_t i = 0; i < ops.size() && use < 0; ++i) {
      const json::Value& u = ops[i];
      if (u.at("type").str() != "BloomFilterUsePOp") continue;
      const std::string un = u.at("name").str();
      cols = u.contains("bloomFilterColumns") ? u.str_list("bloomFilterColumns")
                                              : std::vector<std::string>{u.at("bloomFilterColumn").str()};
      crs = u.str_list("creators");
      if (crs.empty()) crs = creators[un];
      if (crs.size() != cols.size()) continue;
      auto cons = u.str_list("consumers");
      if (cons.size() != 1) continue;
      const int j = index_of(cons[0]);
      if (j < 0) continue;
      const json::Value& J = ops[j];
      if (J.at("type").str() != "HashJoinArrowPOp" || J.get_str("joinType", "INNER") != "INNER" ||
          J.contains("buildKeys") || !J.contains("buildKey"))
        continue;
      // the use must be the build side's only producer: the build tests its
      // filters on every build row, and rows from another producer were
      // never filtered
      auto bp = J.str_list("buildProducers"), pp = J.str_list("probeProducers");
      if (bp != std::vector<std::string>{un} || std::find(pp.begin(), pp.end(), un) != pp.end()) continue;
      const std::string key = J.at("buildKey").str();
      bool on_key = true;
      for (auto& c : cols) on_key &= c == key;
      const size_t have = J.contains("buildFilters") ? J.at("buildFilters").array().size() : 0;
      if (!on_key || have + cols.size() > static_cast<size_t>(kJoinBuildFiltersMax)) continue;
      use = static_cast<int>(i);
      join = j;
    }
    if (use < 0) break;
    const std::string un = ops[use].at("name").str(), jn = ops[join].at("name").str();
    std::vector<std::string> data;  // the use's data producers
    for (auto& p : producers[un])
      if (std::find(crs.begin(), crs.end(), p) == crs.end()) data.push_back(p);
    for (auto& o : ops) {
      if (o.at("type").str() != "BloomFilterCreatePOp" || o.contains("dataConsumers")) continue;
      auto uses = o.str_list("bloomFilterUsePOps");
      std::vector<std::string> dc;
      for (auto& c : o.str_list("consumers"))
        if (std::find(uses.begin(), uses.end(), c) == uses.end()) dc.push_back(c);
      jset(o, "dataConsumers", jlist(dc));
    }
    for (auto& o : ops) {
      if (&o == &ops[use]) continue;
      const bool is_creator = std::find(crs.begin(), crs.end(), o.at("name").str()) != crs.end();
      for (const char* key : {"consumers", "bloomFilterUsePOps", "dataConsumers", "buildProducers"}) {
        const std::string k = key;
        rewrite_names(o, key, [&](const std::string& x, std::vector<std::string>& out) {
          if (x != un) return false;
          if (k == "buildProducers") out = data;
          else if (!(k == "consumers" && is_creator)) out.push_back(jn);  // a creator's filter goes by "bloomFilterUsePOps"
          return true;
        });
      }
    }
    json::Value filters;
    if (ops[join].contains("buildFilters")) filters = ops[join].at("buildFilters");
    else filters.kind = json::Value::Array;
    for (size_t k = 0; k < cols.size(); ++k) {
      json::Value f;
      f.kind = json::Value::Object;
      jset(f, "column", jstr(cols[k]));
      jset(f, "creator", jstr(crs[k]));
      filters.a.push_back(f);
    }
    jset(ops[join], "buildFilters", filters);
    ops.erase(ops.begin() + use);
  }
}

// Pipeline fusion: BloomFilterCreatePOps over the same rows become one
// operator that builds all their filters in one pass (bloom_build_many):
// a creator whose only ordinary consumer is another creator, that one's
// only producer (a chain, each forwarding the rows to the next), or a
// creator with no ordinary consumer and another with the same single
// producer (siblings). The fused operator keeps the second one's name and
// ordinary consumers; each filter keeps its creator's name as its origin,
// which its receivers know it by, and goes to the same receivers. Results
// are unchanged: every filter is built from the same rows as before.
void fuse_creator_chains(std::vector<json::Value>& ops) {
  auto is_creator = [](const json::Value& o) { return o.at("type").str() == "BloomFilterCreatePOp"; };
  auto index_of = [&](const std::string& name) {
    for (size_t i = 0; i < ops.size(); ++i)
      if (ops[i].at("name").str() == name) return static_cast<int>(i);
    return -1;
  };
  auto filters_of = [](const json::Value& c) {
    if (c.contains("filters")) return c.at("filters").array();
    json::Value f;
    f.kind = json::Value::Object;
    jset(f, "origin", c.at("name"));
    jset(f, "bloomFilterColumn", c.at("bloomFilterColumn"));
    for (const char* k : {"bitsPerKey", "numHashes"})
      if (c.contains(k)) jset(f, k, c.at(k));
    jset(f, "bloomFilterUsePOps", jlist(c.str_list("bloomFilterUsePOps")));
    return std::vector<json::Value>{f};
  };
  auto data_consumers_of = [](const json::Value& c) {
    if (c.contains("dataConsumers")) return c.str_list("dataConsumers");
    auto uses = c.str_list("bloomFilterUsePOps");
    std::vector<std::string> dc;
    for (auto& x : c.str_list("consumers"))
      if (std::find(uses.begin(), uses.end(), x) == uses.end()) dc.push_back(x);
    return dc;
  };
  for (;;) {
    std::map<std::string, std::vector<std::string>> producers;
    for (auto& o : ops)
      for (auto& c : o.str_list("consumers")) producers[c].push_back(o.at("name").str());
    int a = -1, b = -1;
    for (size_t i = 0; i < ops.size() && a < 0; ++i) {
      if (!is_creator(ops[i])) continue;
      const std::string an = ops[i].at("name").str();
      const auto dc = data_consumers_of(ops[i]);
      const size_t na = filters_of(ops[i]).size();
      if (dc.size() == 1) {  // a chain
        const int j = index_of(dc[0]);
        if (j >= 0 && is_creator(ops[j]) && producers[dc[0]] == std::vector<std::string>{an} &&
            na + filters_of(ops[j]).size() <= static_cast<size_t>(kBloomBuildManyMax)) {
          a = static_cast<int>(i);
          b = j;
        }
      } else if (dc.empty() && producers[an].size() == 1) {  // siblings
        for (size_t j = 0; j < ops.size(); ++j) {
          if (j == i || !is_creator(ops[j]) || producers[ops[j].at("name").str()] != producers[an]) continue;
          if (na + filters_of(ops[j]).size() > static_cast<size_t>(kBloomBuildManyMax)) continue;
          a = static_cast<int>(i);
          b = static_cast<int>(j);
          break;
        }
      }
    }
    if (a < 0) break;
    const std::string an = ops[a].at("name").str(), bn = ops[b].at("name").str();
    json::Value filters;
    filters.kind = json::Value::Array;
    filters.a = filters_of(ops[a]);
    for (auto& f : filters_of(ops[b])) filters.a.push_back(f);
    std::vector<std::string> uses, cons;
    for (auto& f : filters.a)
      for (auto& u : f.str_list("bloomFilterUsePOps"))
        if (std::find(uses.begin(), uses.end(), u) == uses.end()) uses.push_back(u);
    for (const json::Value* o : {&ops[a], &ops[b]})
      for (auto& c : o->str_list("consumers"))
        if (c != bn && std::find(cons.begin(), cons.end(), c) == cons.end()) cons.push_back(c);
    json::Value fused;
    fused.kind = json::Value::Object;
    jset(fused, "type", jstr("BloomFilterCreatePOp"));
    jset(fused, "name", jstr(bn));
    jset(fused, "filters", filters);
    jset(fused, "bloomFilterUsePOps", jlist(uses));
    jset(fused, "dataConsumers", jlist(data_consumers_of(ops[b])));
    jset(fused, "consumers", jlist(cons));
    ops[b] = fused;
    auto to_bn = [&](const std::string& x, std::vector<std::string>& out) {
      if (x != an) return false;
      out.push_back(bn);
      return true;
    };
    for (auto& o : ops)
      for (const char* key : {"consumers", "bloomFilterUsePOps", "buildProducers", "probeProducers", "dataConsumers"})
        rewrite_names(o, key, to_bn);
    ops.erase(ops.begin() + a);
  }
}

// Pipeline fusion: a chain of inner HashJoinArrowPOps in which each join's
// only consumer is the next join, which takes it as its only probe producer,
// becomes one HashJoinChainPOp (the joins in order, each with its build
// producers, keys, load factor and projection). The fused operator keeps the
// last join's name, so every reference to the chain's end stays valid, and
// every producer that sent to an earlier join now sends to it. Results are
// unchanged: the fused operator builds the same tables and emits the last
// join's rows.
void fuse_join_chains(std::vector<json::Value>& ops) {
  auto is_join = [](const json::Value& o) {
    return o.at("type").str() == "HashJoinArrowPOp" && o.get_str("joinType", "INNER") == "INNER" &&
           !o.contains("buildKeys");  // multi-column keys join one at a time
  };
  auto index_of = [&](const std::string& name) {
    for (size_t i = 0; i < ops.size(); ++i)
      if (ops[i].at("name").str() == name) return static_cast<int>(i);
    return -1;
  };
  // the join that follows ops[i] in a chain, or -1
  auto next_of = [&](size_t i) {
    if (!is_join(ops[i])) return -1;
    auto cons = ops[i].str_list("consumers");
    if (cons.size() != 1) return -1;
    const int j = index_of(cons[0]);
    if (j < 0 || !is_join(ops[j])) return -1;
    if (ops[j].str_list("probeProducers") != std::vector<std::string>{ops[i].at("name").str()}) return -1;
    auto bp = ops[j].str_list("buildProducers");
    if (std::find(bp.begin(), bp.end(), ops[i].at("name").str()) != bp.end()) return -1;
    return j;
  };
  for (;;) {
    // each join's chain successor, then the first join of a chain: a join no
    // other join feeds as its chain successor
    std::vector<int> nxt(ops.size());
    std::vector<bool> fed(ops.size(), false);
    for (size_t i = 0; i < ops.size(); ++i) {
      nxt[i] = next_of(i);
      if (nxt[i] >= 0) fed[static_cast<size_t>(nxt[i])] = true;
    }
    int head = -1;
    for (size_t i = 0; i < ops.size() && head < 0; ++i)
      if (nxt[i] >= 0 && !fed[i]) head = static_cast<int>(i);
    if (head < 0) break;
    std::vector<int> chain{head};
    while (static_cast<int>(chain.size()) < kJoinChainMax) {
      const int j = nxt[static_cast<size_t>(chain.back())];
      if (j < 0) break;
      chain.push_back(j);
    }
    if (chain.size() < 2) break;
    json::Value fused;
    fused.kind = json::Value::Object;
    jset(fused, "type", jstr("HashJoinChainPOp"));
    jset(fused, "name", ops[chain.back()].at("name"));
    json::Value joins;
    joins.kind = json::Value::Array;
    std::set<std::string> absorbed;
    for (int i : chain) {
      const json::Value& o = ops[i];
      json::Value j;
      j.kind = json::Value::Object;
      for (const char* k : {"name", "buildProducers", "buildKey", "probeKey", "loadFactor", "projectColumnNames", "joinType",
                            "buildFilters"})
        if (o.contains(k)) jset(j, k, o.at(k));
      joins.a.push_back(j);
      absorbed.insert(o.at("name").str());
    }
    jset(fused, "joins", joins);
    jset(fused, "probeProducers", ops[chain.front()].at("probeProducers"));
    jset(fused, "consumers", jlist(ops[chain.back()].str_list("consumers")));
    const std::string last = ops[chain.back()].at("name").str();
    std::vector<json::Value> kept;
    kept.reserve(ops.size());
    for (size_t i = 0; i < ops.size(); ++i) {
      if (absorbed.count(ops[i].at("name").str())) {
        if (static_cast<int>(i) == chain.back()) kept.push_back(std::move(fused));
        continue;
      }
      json::Value o = std::move(ops[i]);
      auto to_last = [&](const std::string& x, std::vector<std::string>& out) {
        if (!absorbed.count(x)) return false;
        out.push_back(last);
        return true;
      };
      for (const char* key : {"consumers", "bloomFilterUsePOps", "buildProducers", "probeProducers", "dataConsumers"})
        rewrite_names(o, key, to_last);
      if (json::Value* fl = jfind(o, "filters"))  // a fused creator's receivers, filter by filter
        for (auto& f : fl->a) rewrite_names(f, "bloomFilterUsePOps", to_last);
      kept.push_back(std::move(o));
    }
    ops = std::move(kept);
  }
}

json::Value fuse_pipelines(const json::Value& plan) {
  json::Value out = plan;  // the passes rewrite the copy's operator list in place
  json::Value* ops_v = jfind(out, "ops");
  if (ops_v == nullptr || ops_v->kind != json::Value::Array) return out;
  fuse_bloom_chains(ops_v->a);
  fuse_build_filters(ops_v->a);
  fuse_creator_chains(ops_v->a);
  fuse_join_chains(ops_v->a);
  return out;
}

std::unique_ptr<Execution> build_execution(const json::Value& plan_in, cudaStream_t stream) {
  const bool fuse = plan_in.get_bool("fusePipelines", true);
  const json::Value plan = fuse ? fuse_pipelines(plan_in) : plan_in;
  auto ex = std::make_unique<Execution>(stream);
  for (auto& o : plan.at("ops").array()) ex->add(make_op(o, ex.get()));
  for (auto& o : plan.at("ops").array()) {
    // BloomFilterCreatePOp's use-ops are consumers too (they wait for its COMPLETE).
    if (o.at("type").str() == "BloomFilterCreatePOp")
      for (auto& u : o.str_list("bloomFilterUsePOps")) {
        auto& cons = ex->op(o.at("name").str())->consumers();
        if (std::find(cons.begin(), cons.end(), u) == cons.end()) cons.push_back(u);
      }
  }
  ex->connect();
  const int64_t streams = plan.get_int("streams", kDefaultPlanStreams);
  if (streams < 1 || streams > 16) fail(GFPDB_EINVAL, "\"streams\" must be in [1, 16]");
  ex->setStreams(static_cast<int>(streams));
  return ex;
}

void validate_plan(const json::Value& plan) {
  // Host-only structural check: operators parse, names are unique, every
  // consumer exists and there is exactly one CollatePOp.
  std::set<std::string> names;
  int collates = 0;
  for (auto& o : plan.at("ops").array()) {
    const std::string name = o.at("name").str();
    if (!names.insert(name).second) fail(GFPDB_EINVAL, "duplicate operator name '" + name + "'");
    if (o.at("type").str() == "CollatePOp") ++collates;
    (void)make_op(o, nullptr);
  }
  for (auto& o : plan.at("ops").array())
    for (auto& c : o.str_list("consumers"))
      if (!names.count(c)) fail(GFPDB_EINVAL, "operator '" + o.at("name").str() + "' sends to unknown '" + c + "'");
  if (collates != 1) fail(GFPDB_EINVAL, "a plan needs exactly one CollatePOp");
}

}  // namespace gfpdb::pop
