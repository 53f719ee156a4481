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
};

struct gfpdb_hashjoin {
  int32_t join_type = GFPDB_JOIN_INNER;
  std::string build_key, probe_key;
  std::vector<std::string> needed;
  bool all_columns = true;
  double load_factor = 0.5;
  std::vector<gfpdb::TupleSetPtr> build;
  gfpdb::JoinTable table;
  bool built = false;
};

struct gfpdb_group {
  std::shared_ptr<gfpdb::GroupTable> table;
};
