// Definitions of the opaque handles declared in include/gfpdb.h.
#pragma once

#include <string>
#include <vector>

#include "../kernels/launch.h"

struct gfpdb_filter {
  gfpdb::CompiledPredicate pred;
};

struct gfpdb_bloom {
  gfpdb::BloomPtr bloom;
  int32_t key_columns = 1;  // the filter holds the composite of this many key columns
};

struct gfpdb_hashjoin {
  int32_t join_type = GFPDB_JOIN_INNER;
  std::vector<std::string> build_keys, probe_keys;
  std::vector<std::string> needed;
  bool all_columns = true;
  double load_factor = 0.5;
  std::vector<gfpdb::TupleSetPtr> build;
  gfpdb::JoinTable table;
  std::vector<gfpdb::Field> probe_fields;  // from the first probed batch
  bool built = false;
};

struct gfpdb_group {
  std::shared_ptr<gfpdb::GroupTable> table;
  // the spec, to start a fresh table on clear
  std::vector<std::string> group_cols;
  std::vector<gfpdb::GroupAggregate> aggs;
  int64_t hint = 0;
};
