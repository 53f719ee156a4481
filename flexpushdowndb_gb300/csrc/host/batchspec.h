// The JSON form of a batched star query (documented with gfpdb_star_batch in
// include/gfpdb.h), shared by the C ABI and the request server.
#pragma once

#include <string>
#include <vector>

#include "../kernels/launch.h"
#include "json.h"

namespace gfpdb {

// Fills `sp` from the spec; "queries" is optional (a template for the server,
// whose queries arrive one per request).
void parse_star_batch_spec(const json::Value& spec, StarBatchSpec& sp);

// The columns of each table the batch reads: (table, column) pairs.
std::vector<std::pair<std::string, std::string>> star_batch_columns(const StarBatchSpec& sp);

// Captures b.run() as a CUDA graph (b prepared). Returns nullptr when the
// capture fails (the caller then runs b.run() directly); *kernels gets the
// launches per replay.
cudaGraphExec_t capture_star_batch(StarBatch& b, uint64_t* kernels);

// Canonical text of a JSON value (object keys in their given order).
std::string json_dump(const json::Value& v);

}  // namespace gfpdb
