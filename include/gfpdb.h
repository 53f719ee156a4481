/*
 * gfpdb — C ABI of the GB300-native relational hot path (sm_103a).
 *
 * Every entry point is a plain C function over the Arrow C Data / C Device
 * Data Interface (gfpdb_arrow.h): plain pointers, sizes and status codes, no
 * C++ or torch types. Each one replaces one kernel seam of the reference's
 * fpdb-executor physical operators; the comment above it names the reference
 * interface (file:line) it stands in for.
 *
 * Conventions
 *  - Return value: GFPDB_OK (0) or a GFPDB_E* code. The message of the last
 *    failure on the calling thread is returned by gfpdb_last_error(); this is
 *    the C rendering of the reference's tl::expected<T, std::string> results.
 *  - A TupleSet crosses the boundary as (ArrowSchema "+s", ArrowDeviceArray
 *    whose struct array has one child per column). Input arrays may live in
 *    device memory (ARROW_DEVICE_CUDA) or in host memory (ARROW_DEVICE_CPU /
 *    ARROW_DEVICE_CUDA_HOST); host inputs are copied to the device on the
 *    given stream. Outputs are device arrays owned by the library until the
 *    caller invokes their release callbacks (Arrow spec semantics).
 *  - Supported column formats: "i" int32, "l" int64, "tdD" date32, "g"
 *    float64, "u" utf8. Decimals are carried as int64 cents.
 *  - `stream` is a cudaStream_t (NULL = the legacy default stream). Calls are
 *    reentrant across streams. There is no CPU fallback: every compute entry
 *    point launches CUDA kernels and fails with GFPDB_ECUDA when no device is
 *    usable.
 */
#ifndef GFPDB_H
#define GFPDB_H

#include <stdint.h>
#include "gfpdb_arrow.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GFPDB_OK 0
#define GFPDB_EINVAL 1        /* bad argument, schema, plan or expression */
#define GFPDB_ECUDA 2         /* CUDA runtime error (no device, launch failure) */
#define GFPDB_EDEVICE 3       /* a kernel raised its device error word */
#define GFPDB_ETIMEDOUT 4     /* a bounded device-side wait gave up */
#define GFPDB_ENOMEM 5        /* device allocation failed or HBM budget exceeded */
#define GFPDB_EUNSUPPORTED 6  /* valid request outside what this build implements */

/* Join types, numbered like fpdb::plan::prephysical::JoinType. */
#define GFPDB_JOIN_INNER 0
#define GFPDB_JOIN_LEFT 1
#define GFPDB_JOIN_RIGHT 2
#define GFPDB_JOIN_FULL 3
#define GFPDB_JOIN_LEFT_SEMI 4
#define GFPDB_JOIN_RIGHT_SEMI 5

typedef struct gfpdb_filter gfpdb_filter;
typedef struct gfpdb_bloom gfpdb_bloom;
typedef struct gfpdb_hashjoin gfpdb_hashjoin;
typedef struct gfpdb_group gfpdb_group;

/* ---------------------------------------------------------------- runtime */

/* Message of the last failed call on this thread ("" if none). */
const char* gfpdb_last_error(void);

/* ABI version (major * 10000 + minor * 100 + patch). */
int32_t gfpdb_version(void);

/* Select the CUDA device for this thread and set up its memory pool.
 * Idempotent. Replaces nothing in the reference (its operators are CPU-only);
 * it is the device-side counterpart of Executor::start
 * (fpdb-executor/src/Executor.cpp:40-65). */
int32_t gfpdb_device_init(int32_t device);

/* Number of kernels this library has launched in this process. */
uint64_t gfpdb_kernel_launch_count(void);

/* Bytes of device memory the calling thread has taken from the library's
 * allocator so far (each request rounded up to 256 bytes). A diagnostic with
 * no counterpart in the reference: a caller checks with it that a call
 * allocated nothing, or how much a plan's first run allocated. */
int64_t gfpdb_thread_device_alloc_bytes(void);

/* Stream-ordered copies between host and device memory, for callers that
 * hold raw device buffers (kind: 1 = host->device, 2 = device->host,
 * 3 = device->device). Synchronous when stream is NULL. */
int32_t gfpdb_memcpy(void* dst, const void* src, int64_t n_bytes, int32_t kind, void* stream);

/* The layout of an exported TupleSet (an output of this library), for a
 * caller that copies it out in one pass: its row count, where its buffers
 * live (ARROW_DEVICE_CPU or ARROW_DEVICE_CUDA), and per column its name and
 * Arrow format string, written into `names` as "name\0format\0" pairs, its
 * values buffer and, for utf8, its offsets buffer (NULL otherwise). Fails
 * with GFPDB_EINVAL when the TupleSet has more than max_columns columns or
 * the names do not fit names_capacity bytes. */
/* (A column with a validity bitmap, an outer join's output, is refused
 * with GFPDB_EUNSUPPORTED: the layout carries values only.) */
int32_t gfpdb_result_layout(const struct ArrowSchema* schema, const struct ArrowDeviceArray* array,
                            int32_t max_columns, int64_t* n_rows, int32_t* n_columns, int32_t* device_type,
                            char* names, int64_t names_capacity, const void** values, const void** offsets);

/* Releases both structures of an exported TupleSet (either may already be
 * released or NULL). */
void gfpdb_result_release(struct ArrowSchema* schema, struct ArrowDeviceArray* array);

/* Page-locked host allocation, so that host inputs can be copied at full
 * link bandwidth. */
int32_t gfpdb_host_alloc(void** ptr, int64_t n_bytes);
int32_t gfpdb_host_free(void* ptr);

/* Wait for all work queued on `stream`. */
int32_t gfpdb_stream_synchronize(void* stream);

/* Kernel timing: while enabled, every kernel launch of the library is
 * bracketed by CUDA events on its own stream, and its algorithmic byte count
 * (input bytes it must read plus output bytes it writes, at row granularity)
 * is recorded. gfpdb_profile_read returns, for one kernel name, the number of
 * launches, their summed event time in milliseconds and their summed
 * algorithmic bytes (it waits for the recorded events). The tracing
 * counterpart of the reference's per-operator timing (SHOW_OP_TIMES,
 * fpdb-executor/src/Execution.cpp:420). */
int32_t gfpdb_profile_enable(int32_t enable);
int32_t gfpdb_profile_reset(void);
int32_t gfpdb_profile_read(const char* kernel_name, int64_t* launches, double* total_ms, double* total_bytes);
/* Names of the kernels recorded since the last reset, '\n'-separated. */
int32_t gfpdb_profile_kernels(char* buf, int64_t buf_len);

/* ----------------------------------------------------------------- filter */

/* Compile a predicate expression tree against a schema.
 * Replaces fpdb::expression::gandiva::Filter::make + Filter::compile
 * (fpdb-expression-gandiva/src/Filter.cpp:227-271): the Gandiva LLVM JIT
 * becomes a lowering to a conjunctive leaf program that the fused selection
 * kernel evaluates. `predicate_json` uses the reference's expression JSON
 * node names (Expression::fromJson, fpdb-expression-gandiva/src/Expression.cpp:52-148). */
int32_t gfpdb_filter_compile(const char* predicate_json, const struct ArrowSchema* schema,
                             gfpdb_filter** out);

/* Evaluate a compiled predicate over one TupleSet and emit the selected rows
 * (input order kept) projected to `project_columns` (all columns when
 * n_project < 0). Replaces Filter::evaluate(const TupleSet&)
 * (fpdb-expression-gandiva/src/Filter.cpp:87-176) as called by
 * FilterPOp::filterTuplesRegular (fpdb-executor/src/physical/filter/FilterPOp.cpp:316-339). */
int32_t gfpdb_filter_evaluate(const gfpdb_filter* filter, const struct ArrowSchema* in_schema,
                              const struct ArrowDeviceArray* in, const char* const* project_columns,
                              int32_t n_project, struct ArrowSchema* out_schema,
                              struct ArrowDeviceArray* out, void* stream);

void gfpdb_filter_free(gfpdb_filter* filter);

/* The filter of gfpdb_filter_evaluate for callers that cannot allocate device
 * memory: engines that own a fixed device arena and budget every byte of HBM
 * themselves, and embedders whose device memory belongs to another runtime's
 * allocator, for whom a cudaMalloc by the library would grow the heap behind
 * their accounting. It has no counterpart in the reference. It allocates
 * nothing: the kernel's scratch (status block, tile ticket, one look-back
 * word per 2048-row tile) lives in a file-scope __device__ array of about
 * 1 MiB that every GPU loading the library keeps until exit, and the caller
 * passes the outputs.
 *  - Input must be device-resident (ARROW_DEVICE_CUDA) and at most
 *    268,435,456 rows; larger inputs are rejected with GFPDB_EINVAL.
 *  - out_columns[j] is a device buffer for project_columns[j] with room for
 *    in->array.length values of that column's width; only fixed-width columns
 *    (int32, int64, date32, float64) without nulls can be outputs.
 *  - The input is checked as gfpdb_filter_evaluate checks it (struct without
 *    nulls, children at least offset + length long with their buffer counts,
 *    no nullable columns); a failed check is GFPDB_EINVAL or
 *    GFPDB_EUNSUPPORTED before any device work.
 *  - *out_num_rows receives the number of selected rows (the call waits for
 *    its stream).
 *  - The first call on a device looks up the array's device address
 *    (cudaGetSymbolAddress); make that first call before any stream capture.
 *  - All calls share the one array, and each call clears the part it uses, so
 *    calls that overlap on the GPU (other streams, other threads) race:
 *    serialise them. */
int32_t gfpdb_filter_evaluate_noalloc(const gfpdb_filter* filter, const struct ArrowSchema* in_schema,
                                      const struct ArrowDeviceArray* in, const char* const* project_columns,
                                      int32_t n_project, void* const* out_columns, int64_t* out_num_rows,
                                      void* stream);

/* ------------------------------------------------------------------ bloom */

/* Build a blocked bloom filter (256-bit blocks, `num_hashes` bits per key set
 * inside one block, sized `bits_per_key` bits per key) over the key of one or
 * more TupleSets: one column, or the composite of n_keys columns (the
 * reference's bloomFilterColumnNames, BloomFilterCreatePOp.cpp:17-22). Replaces BloomFilterCreateArrowKernel::buildBloomFilter
 * (fpdb-executor/src/physical/bloomfilter/BloomFilterCreateArrowKernel.cpp:17-34)
 * and ArrowBloomFilter::build (.../bloomfilter/ArrowBloomFilter.cpp:29-75).
 * Above GFPDB_BLOOM_MAX_INPUT_SIZE keys the filter is marked invalid and every
 * probe passes, as BLOOM_FILTER_MAX_INPUT_SIZE does in the reference
 * (fpdb-executor/include/fpdb/executor/physical/Globals.h:55,
 * .../bloomfilter/BloomFilterUseKernel.cpp:17-19). */
#define GFPDB_BLOOM_MAX_INPUT_SIZE 20000000
int32_t gfpdb_bloom_create(const struct ArrowSchema* schema,
                           const struct ArrowDeviceArray* const* batches, int32_t n_batches,
                           const char* const* key_columns, int32_t n_keys, int32_t bits_per_key,
                           int32_t num_hashes, gfpdb_bloom** out, void* stream);

/* Keep the rows whose key may be in the filter; all columns are kept. The
 * key columns (1 to 8, as many as the filter was built over) are named in
 * key_columns. Replaces BloomFilterUseKernel::filter(tupleSet, bloomFilter,
 * columnNames) (fpdb-executor/src/physical/bloomfilter/BloomFilterUseKernel.cpp:12-32). */
int32_t gfpdb_bloom_use(const gfpdb_bloom* bloom, const struct ArrowSchema* in_schema,
                        const struct ArrowDeviceArray* in, const char* const* key_columns, int32_t n_keys,
                        struct ArrowSchema* out_schema, struct ArrowDeviceArray* out, void* stream);

/* Filter structure, for tests and for shipping a filter to another device:
 * block count, keys inserted, whether the filter is valid, and the device
 * address of its num_blocks * 8 uint32 words. */
int32_t gfpdb_bloom_info(const gfpdb_bloom* bloom, int64_t* num_blocks, int64_t* num_keys,
                         int32_t* valid, int32_t* num_hashes, const void** device_blocks);

void gfpdb_bloom_free(gfpdb_bloom* bloom);

/* ------------------------------------------------------------------ shuffle */

/* Hash-partition the rows of a TupleSet into num_slots slots (1 to 1024) by
 * n_keys key columns (1 to 8; integer, date32 or utf8): the output holds
 * every input row once, slot by slot, input order kept within a slot; slot i
 * is rows [slot_offsets[i], slot_offsets[i+1]) (num_slots + 1 entries
 * written). Equal keys always share a slot; integer keys hash by value, so
 * int32 and int64 columns of equal values agree.
 * Replaces ShuffleKernel2::shuffle(columnNames, numSlots, tupleSet)
 * (fpdb-executor/src/physical/shuffle/ShuffleKernel2.cpp:28-125), whose
 * vector of per-slot TupleSets is the output sliced at slot_offsets. */
int32_t gfpdb_shuffle(const struct ArrowSchema* in_schema, const struct ArrowDeviceArray* in,
                      const char* const* key_columns, int32_t n_keys, int64_t num_slots,
                      struct ArrowSchema* out_schema, struct ArrowDeviceArray* out, int64_t* slot_offsets,
                      void* stream);

/* ----------------------------------------------- fused scan (filter+bloom) */

/* One fused pass over a TupleSet: an optional compiled predicate AND a chain
 * of bloom probes, followed by stable compaction and projection. This is the
 * GPU form of a FilterPOp followed by a chain of BloomFilterUsePOps
 * (FilterPOp.cpp:316-339; BloomFilterUsePOp.cpp:116-142), which the reference
 * runs as separate passes. `filter` may be NULL; n_blooms may be 0. */
int32_t gfpdb_select(const gfpdb_filter* filter, int32_t n_blooms, const gfpdb_bloom* const* blooms,
                     const char* const* bloom_key_columns, const struct ArrowSchema* in_schema,
                     const struct ArrowDeviceArray* in, const char* const* project_columns,
                     int32_t n_project, struct ArrowSchema* out_schema,
                     struct ArrowDeviceArray* out, void* stream);

/* -------------------------------------------------------------- hash join */

/* Create a hash join on n_keys key columns per side (1 to 8; build_keys[i]
 * matches probe_keys[i], HashJoinPredicate(leftColumnNames,
 * rightColumnNames), fpdb-executor/include/fpdb/executor/physical/join/hashjoin/HashJoinPredicate.h:25-26;
 * several columns are joined on a composite of their hashes and the rows
 * whose key columns differ are then dropped, so the result is exact).
 * join_type is the reference's JoinType (GFPDB_JOIN_*,
 * fpdb-plan/include/fpdb/plan/prephysical/JoinType.h:13-20) with its
 * HashJoinArrowKernel meaning (HashJoinArrowKernel.cpp:164-195): LEFT keeps
 * every build row, RIGHT every probe row, FULL both (the missing side's
 * columns null: a validity bitmap in buffers[0], null_count -1), LEFT_SEMI
 * emits the build rows with a match (build columns only), RIGHT_SEMI the
 * probe rows with a match (probe columns only). Non-inner joins take one
 * integer key column per side; the rows decided by the build side (LEFT /
 * FULL unmatched, LEFT_SEMI) come from gfpdb_hashjoin_finish.
 * Output columns are the probe side's needed columns followed by the build
 * side's, as HashJoinArrowKernel::makeOutputSchema orders them
 * (fpdb-executor/src/physical/join/hashjoin/HashJoinArrowKernel.cpp:148-162).
 * `needed_columns` NULL / n_needed < 0 keeps every column.
 * Replaces HashJoinArrowKernel::make (HashJoinArrowKernel.h:48-54). */
int32_t gfpdb_hashjoin_create(int32_t join_type, const char* const* build_keys, const char* const* probe_keys,
                              int32_t n_keys, const char* const* needed_columns, int32_t n_needed,
                              double load_factor, gfpdb_hashjoin** out);

/* Append a build-side TupleSet. Replaces HashJoinArrowKernel::joinBuildTupleSet
 * (HashJoinArrowKernel.cpp:35-63). */
int32_t gfpdb_hashjoin_put_build(gfpdb_hashjoin* join, const struct ArrowSchema* schema,
                                 const struct ArrowDeviceArray* batch, void* stream);

/* All build input has arrived: build the open-addressing table.
 * Replaces HashJoinArrowKernel::finalizeInput(true) (HashJoinArrowKernel.cpp:95-124). */
int32_t gfpdb_hashjoin_finalize_build(gfpdb_hashjoin* join, void* stream);

/* Probe one TupleSet against the built table and emit the joined rows.
 * Replaces HashJoinArrowKernel::joinProbeTupleSet + getOutputBuffer
 * (HashJoinArrowKernel.cpp:65-93). */
int32_t gfpdb_hashjoin_probe(gfpdb_hashjoin* join, const struct ArrowSchema* schema,
                             const struct ArrowDeviceArray* batch, struct ArrowSchema* out_schema,
                             struct ArrowDeviceArray* out, void* stream);

/* Build-table statistics: rows, slots, longest probe run seen while building. */
/* Every probe batch is in: emit the rows the build side decides (the
 * unmatched build rows with null probe columns for LEFT and FULL, the
 * matched build rows for LEFT_SEMI; no rows for the other types), as
 * HashJoinArrowKernel::finalizeInput on the probe side flushes Arrow's join
 * (HashJoinArrowKernel.cpp:100-116). The probe columns' types come from the
 * probed batches (probe_schema when none was probed; may be NULL). */
int32_t gfpdb_hashjoin_finish(gfpdb_hashjoin* join, const struct ArrowSchema* probe_schema,
                              struct ArrowSchema* out_schema, struct ArrowDeviceArray* out, void* stream);

int32_t gfpdb_hashjoin_info(const gfpdb_hashjoin* join, int64_t* build_rows, int64_t* capacity,
                            int64_t* max_probe);

/* Drop the build input and the table, so the join can take a new build side.
 * Replaces HashJoinArrowKernel::clear (HashJoinArrowKernel.h:56, the
 * PhysicalOp::clear seam, fpdb-executor/include/fpdb/executor/physical/PhysicalOp.h:84). */
int32_t gfpdb_hashjoin_clear(gfpdb_hashjoin* join);

void gfpdb_hashjoin_free(gfpdb_hashjoin* join);

/* --------------------------------------------------------------- group-by */

/* Create a hash group-by from a JSON spec:
 *   {"groupColumnNames": ["a", ...],
 *    "aggregates": [{"function": "SUM"|"COUNT"|"MIN"|"MAX"|"AVG",
 *                    "name": "out", "expr": <expression JSON, absent for count(*)>}],
 *    "groupsHint": N}
 * Output columns are the group columns followed by the aggregates in the
 * given order (GroupArrowKernel::makeOutputSchema,
 * fpdb-executor/src/physical/group/GroupArrowKernel.cpp:156-200). SUM over
 * integers is an int64 two's-complement (wrapping) sum, COUNT an int64, as
 * Arrow's hash_sum / hash_count (Sum.cpp:63-74, Count.cpp:91-104). */
int32_t gfpdb_group_create(const char* group_spec_json, gfpdb_group** out);

/* Fold one TupleSet into the group table. Replaces GroupAbstractKernel::group
 * (fpdb-executor/include/fpdb/executor/physical/group/GroupAbstractKernel.h:32)
 * as GroupArrowKernel::group implements it (GroupArrowKernel.cpp:16-39). */
int32_t gfpdb_group_update(gfpdb_group* group, const struct ArrowSchema* schema,
                           const struct ArrowDeviceArray* batch, void* stream);

/* Emit one row per group. Replaces GroupAbstractKernel::finalise
 * (GroupAbstractKernel.h:39; GroupArrowKernel.cpp:41-68). */
int32_t gfpdb_group_finalize(gfpdb_group* group, struct ArrowSchema* out_schema,
                             struct ArrowDeviceArray* out, void* stream);

/* Drop every group, so the same spec starts over. Replaces
 * GroupAbstractKernel::clear
 * (fpdb-executor/include/fpdb/executor/physical/group/GroupAbstractKernel.h:44). */
int32_t gfpdb_group_clear(gfpdb_group* group);

void gfpdb_group_free(gfpdb_group* group);

/* ---------------------------------------------------------------- Parquet */

/* Read columns of a Parquet file held in host memory (`file`, n_bytes):
 * `columns` names them (all when n_columns < 0), in that order; with
 * start_pos <= end_pos only the row groups whose first column chunk starts
 * within [start_pos, end_pos] (pass 0, -1 for the whole file). Flat schemas
 * of INT32 (DATE annotated: date32), INT64, DOUBLE and BYTE_ARRAY (utf8)
 * columns, required or optional without nulls; PLAIN and dictionary
 * encodings; data pages v1 and v2; uncompressed or snappy. The footer and
 * page headers are read on the host, the pages decompressed and decoded on
 * the device. Replaces ParquetReader::read / readRange
 * (fpdb-tuple/src/parquet/ParquetReader.cpp:12-120) under
 * LocalParquetReader (fpdb-tuple/src/parquet/LocalParquetReader.cpp:25-59). */
int32_t gfpdb_parquet_read(const void* file, int64_t n_bytes, const char* const* columns, int32_t n_columns,
                           int64_t start_pos, int64_t end_pos, struct ArrowSchema* out_schema,
                           struct ArrowDeviceArray* out, void* stream);

/* The layout of a Parquet file held in host memory (host only, no CUDA
 * calls), as JSON: {"numRows", "columns": [{"name", "type", "physicalType",
 * "required"}], "rowGroups": [{"offset", "rows"}], "chunks": [{"begin",
 * "end"}], "pages": [{"column", "chunk", "pageType", "encoding", "codec",
 * "offset", "compressedBytes", "uncompressedBytes", "numValues",
 * "firstRow"}]} for the columns and row groups gfpdb_parquet_read with the
 * same arguments reads (a row group's offset is the file position of its
 * first column chunk, which start_pos / end_pos select it by; the reference
 * splits a file into scan ranges the same way, ParquetReader::readRange,
 * fpdb-tuple/src/parquet/ParquetReader.cpp:44-77). Files the reader refuses
 * are refused here with the same error. Written into out_json when capacity
 * holds it; *needed is its size with the terminating zero. */
int32_t gfpdb_parquet_layout(const void* file, int64_t n_bytes, const char* const* columns, int32_t n_columns,
                             int64_t start_pos, int64_t end_pos, char* out_json, int64_t capacity, int64_t* needed);

/* The same over a file of the local file system (LocalParquetReader::read). */
int32_t gfpdb_parquet_read_file(const char* path, const char* const* columns, int32_t n_columns, int64_t start_pos,
                                int64_t end_pos, struct ArrowSchema* out_schema, struct ArrowDeviceArray* out,
                                void* stream);

/* -------------------------------------------------------------------- CSV */

/* Parse delimiter-separated text into typed columns. `target_schema` ("+s")
 * names and types every field of a line in file order; `columns` selects the
 * fields to emit (all when n_columns < 0). Field types: int32, int64, date32
 * (YYYY-MM-DD), utf8, and int64 with metadata-free format "l" for decimals
 * when the schema child's name ends with no marker: decimal(15,2) text is
 * selected by giving the child the format "d:15,2" and is emitted as int64
 * cents. `text` may be host or device memory (text_device_type).
 * Replaces CSVReader::read(columnNames) (fpdb-tuple/src/csv/CSVReader.cpp:15-21)
 * and its SIMD parser (CSVToArrowSIMDChunkParser.cpp:183-409). */
int32_t gfpdb_csv_read(const void* text, int64_t n_bytes, int32_t text_device_type, char delimiter,
                       int32_t has_header, const struct ArrowSchema* target_schema,
                       const char* const* columns, int32_t n_columns,
                       struct ArrowSchema* out_schema, struct ArrowDeviceArray* out, void* stream);

/* -------------------------------------------------------- plan execution */

typedef struct gfpdb_exec_stats {
  int64_t elapsed_ns;        /* host wall time of the call */
  int64_t kernel_launches;   /* kernels launched by this call */
  int64_t h2d_bytes;         /* host->device bytes copied by this call */
  int64_t d2h_bytes;         /* device->host bytes copied by this call */
  int64_t num_ops;           /* physical operators in the plan */
  int64_t messages;          /* messages delivered between operators */
  int64_t device_ns;         /* replay of a captured plan: device time from the
                                start of the plan graph to the end of its result
                                copy (CUDA events); 0 for other runs */
} gfpdb_exec_stats;

/* Run a physical plan of the reference's operators (TableScanPOp, CsvScanPOp,
 * FilterPOp, BloomFilterCreatePOp, BloomFilterUsePOp, HashJoinArrowPOp,
 * GroupPOp, AggregatePOp, ProjectPOp, LimitSortPOp, CollatePOp) on one GPU,
 * delivering START / TUPLESET /
 * BLOOM_FILTER / COMPLETE messages between them in the reference's protocol,
 * and return the CollatePOp's TupleSet. Input tables are named; host tables
 * are copied to the device by their scan operator. With result_to_host != 0
 * the result is returned in host memory.
 * Replaces Executor::execute(PhysicalPlan) (fpdb-executor/src/Executor.cpp:87-122)
 * driving Execution::execute (fpdb-executor/src/Execution.cpp:44-280). */
int32_t gfpdb_execute_plan(const char* plan_json, int32_t n_tables, const char* const* table_names,
                           const struct ArrowSchema* const* schemas,
                           const struct ArrowDeviceArray* const* arrays, int32_t result_to_host,
                           struct ArrowSchema* out_schema, struct ArrowDeviceArray* out,
                           gfpdb_exec_stats* stats, void* stream);

/* Prepared plans: a plan bound once to its input tables (which the caller
 * keeps alive and unchanged), for callers that run one query many times
 * (a prepared statement). A run leaves its result in host memory owned by
 * the prepared plan, readable until the next run: gfpdb_prepared_layout
 * describes it (as gfpdb_result_layout does) and its pointers stay valid for
 * every later run that reports the same layout generation. With
 * "cudaGraph" a run after the first two is one graph replay, without the
 * per-call plan lookup and result export of gfpdb_execute_plan. */
typedef struct gfpdb_prepared gfpdb_prepared;
int32_t gfpdb_plan_prepare(const char* plan_json, int32_t n_tables, const char* const* table_names,
                           const struct ArrowSchema* const* schemas,
                           const struct ArrowDeviceArray* const* arrays, gfpdb_prepared** out);
int32_t gfpdb_prepared_run(gfpdb_prepared* plan, gfpdb_exec_stats* stats, void* stream, int64_t* n_rows,
                           int64_t* layout_generation);
/* gfpdb_prepared_run in two halves. launch starts the run on the stream and
 * returns; a replay is then in flight (the first runs, and plans without a
 * graph, complete inside launch). wait finishes it and reports as
 * gfpdb_prepared_run does. Between them the caller may launch other work:
 * two prepared plans of one query, whose texts differ only in a
 * "graphInstance" number (so that each captures its own graph, scratch and
 * result buffers), can run back to back on one stream while the host reads
 * the other's result. One launch at a time per prepared plan; freeing a
 * prepared plan waits for a launch that was not waited for. */
int32_t gfpdb_prepared_launch(gfpdb_prepared* plan, void* stream);
int32_t gfpdb_prepared_wait(gfpdb_prepared* plan, gfpdb_exec_stats* stats, int64_t* n_rows,
                            int64_t* layout_generation);
/* As gfpdb_result_layout for the last run's result, plus its row capacity
 * (the length the buffers can hold: the most rows any run with this layout
 * generation can return). */
int32_t gfpdb_prepared_layout(const gfpdb_prepared* plan, int32_t max_columns, int64_t* capacity,
                              int32_t* n_columns, char* names, int64_t names_capacity, const void** values,
                              const void** offsets);
void gfpdb_prepared_free(gfpdb_prepared* plan);


/* Parse and check a plan without running it (host only, no CUDA calls). */
int32_t gfpdb_plan_validate(const char* plan_json);

/* The plan after pipeline fusion (host only, no CUDA calls): what a run
 * executes when the plan's "fusePipelines" is true (the default). Chains of
 * BloomFilterUsePOps on one input become one BloomFilterUsePOp; a
 * BloomFilterUsePOp whose only consumer is an inner HashJoinArrowPOp on one
 * key column, taking it as its only build producer, with its filters on that key,
 * is folded into the join ("buildFilters": the join build leaves out the
 * rows a filter rejects); chains of inner joins become one HashJoinChainPOp.
 * Writes the fused plan's JSON into out_json when capacity holds it;
 * *needed is its size with the terminating zero. Fields the fused operators
 * carry (a plan may also give them itself):
 *   HashJoinArrowPOp / a HashJoinChainPOp join: "buildFilters":
 *     [{"column": build column, "creator": BloomFilterCreatePOp}], bloom
 *     filters the build side's rows must pass;
 *   BloomFilterCreatePOp: "filters": [{"origin", "bloomFilterColumn",
 *     "bitsPerKey", "numHashes", "bloomFilterUsePOps"}] for several filters
 *     over the same rows (each sent under its origin's name), and
 *     "dataConsumers": the consumers that take its rows (default: every
 *     consumer that is not a filter receiver).
 * The fusion passes replace no reference interface: the reference runs each
 * operator as planned. */
int32_t gfpdb_plan_fuse(const char* plan_json, char* out_json, int64_t capacity, int64_t* needed);

/* Plan the bloom-filter predicate transfer of a join graph (host only), as
 * SmallToLargePredTransOrder::orderPredTrans does
 * (fpdb-executor/src/physical/transform/pred-trans/SmallToLargePredTransOrder.cpp:14-214).
 * spec_json: {"tables": [{"op": <operator producing the table>, "rowCount": n,
 *                         "selectivity": fraction its local filters keep (optional, 1)}],
 *             "joins": [{"left": op, "right": op, "leftColumns": [...], "rightColumns": [...],
 *                        "joinType": "INNER" | "LEFT" | ...}],
 *             "bitsPerKey": 10, "numHashes": 3, "namePrefix": "pt"}
 * Writes {"ops": [BloomFilterCreatePOp / BloomFilterUsePOp operators],
 * "edges": [[producer, consumer], ...], "outputs": {table op: its last
 * operator}} (joins attach to the outputs) into out_json when capacity
 * holds it; *needed is its size with the terminating zero. A join cycle is
 * GFPDB_EINVAL. */
int32_t gfpdb_plan_predicate_transfer(const char* spec_json, char* out_json, int64_t capacity, int64_t* needed);

/* Plans run with "cudaGraph": true and batches run with use_graph are kept,
 * keyed by their text and input buffer addresses, so later calls replay them.
 * They reference the caller's input buffers: clear them before freeing those
 * buffers for good. */
int32_t gfpdb_graph_cache_clear(void);

/* ---------------------------------------------------- batched star queries */

/* Run many star queries that differ only in their dimension filter ranges
 * over one fact table split into partitions, with one launch per stage for
 * all queries and partitions: a dimension pass builds one shared join table
 * per dimension whose rows carry the bitmask of the queries selecting them, a
 * persistent fact pass probes every dimension once per fact row for all
 * queries and aggregates into per-query group tables, and a final pass
 * compacts every query's groups. With use_graph the stages are captured once
 * as a CUDA graph and replayed. Spec JSON:
 *   {"factTables": ["p0", ...],
 *    "dimensions": [{"table": "d1", "key": "d1_pk", "factKey": "fk1", "filterColumn": "d1_f"}, ...],
 *    "groupBy": [{"dimension": 1, "column": "d2_g"}, ...],          (0 to 2)
 *    "aggregates": [{"function": "SUM", "name": "revenue", "columns": ["price_cents", "qty"]},
 *                   {"function": "COUNT", "name": "cnt"}],                  (1 to 4)
 *    "queries": [[[lo, hi], ...one range per dimension...], ...],   (1 to 64)
 *    "probeOrder": [1, 2, 3, 0], "loadFactor": 0.5, "itemsPerThread": 2,
 *    "blocksPerSm": 4, "stages": 3, "groupsHint": 1024}
 * probeOrder (optional) lists every dimension once; without it the smallest
 * dimensions go first. itemsPerThread is 1, 2, 4 or 8; stages (2 to 8) is
 * the depth of each block's foreign-key copy pipeline. Tables may be
 * device-resident or in host memory: a run then first copies every column
 * the batch reads to the device (the dimensions, then the fact partitions in
 * groups, each group's fact pass starting as its copies land; the copied
 * bytes are reported in stats->h2d_bytes), so changes to the host buffers
 * between runs are seen. Pageable host tables run without a graph. Dimensions with
 * dense keys (max - min + 1 within the join table's capacity) are looked up
 * by direct address, the others by hash; the choice is made on the device
 * each run and never changes results. The result has a query_id column, then the group columns, then the
 * aggregates; each query's rows equal that query's single-query plan
 * (the join / group parts of SmallToLargePredTransOrder.cpp's star plans,
 * HashJoinArrowKernel.cpp and GroupArrowKernel.cpp semantics). */
int32_t gfpdb_star_batch(const char* spec_json, int32_t n_tables, const char* const* table_names,
                         const struct ArrowSchema* const* schemas, const struct ArrowDeviceArray* const* arrays,
                         int32_t use_graph, int32_t result_to_host, struct ArrowSchema* out_schema,
                         struct ArrowDeviceArray* out, gfpdb_exec_stats* stats, void* stream);

/* Prepared batches: a batched star query bound once to its tables (which
 * the caller keeps alive and unchanged in place; host tables are re-read by
 * every run), for callers that run the same batch of queries repeatedly.
 * Prepare captures the stages and a pack of the result into page-locked host
 * memory as one CUDA graph; a run is one graph launch (gfpdb_batch_launch
 * returns at once) and a wait for it (gfpdb_batch_wait: status and row
 * count), and the result is read through gfpdb_batch_layout's pointers
 * (query_id, group columns, aggregates; rows [0, n_rows)), valid until the
 * next run. One run at a time per prepared batch: two prepared copies can be
 * launched back to back, each waited for while the other runs. The same
 * kernels as gfpdb_star_batch (above), without its per-call lookup, device
 * synchronizations and result export. */
typedef struct gfpdb_batch gfpdb_batch;
int32_t gfpdb_batch_prepare(const char* spec_json, int32_t n_tables, const char* const* table_names,
                            const struct ArrowSchema* const* schemas, const struct ArrowDeviceArray* const* arrays,
                            gfpdb_batch** out);
int32_t gfpdb_batch_launch(gfpdb_batch* batch, void* stream);
int32_t gfpdb_batch_wait(gfpdb_batch* batch, gfpdb_exec_stats* stats, int64_t* n_rows);
int32_t gfpdb_batch_run(gfpdb_batch* batch, gfpdb_exec_stats* stats, void* stream, int64_t* n_rows);
/* Names and Arrow formats ("name\0format\0" pairs) and host pointers of the
 * result columns (all fixed-width), and the row capacity. */
int32_t gfpdb_batch_layout(const gfpdb_batch* batch, int32_t max_columns, int64_t* capacity, int32_t* n_columns,
                           char* names, int64_t names_capacity, const void** values);
void gfpdb_batch_free(gfpdb_batch* batch);

/* ------------------------------------------------------------ request server */

/* The serving form: a request server on one GPU with an HBM-resident column
 * cache, admission by HBM budget, worker threads on their own CUDA streams and
 * continuous batching of star queries. It stands where the reference's query
 * front end meets fpdb-cache (SegmentCache, fpdb-cache/src/SegmentCache.cpp:21-75,
 * LFU policy fpdb-cache/src/policy/LFUCachingPolicy.cpp; CacheLoadPOp,
 * fpdb-executor/src/physical/cache/CacheLoadPOp.cpp:64-261).
 *
 * Config JSON (every key optional):
 *   {"device": 0, "workers": 4, "hbmBudgetBytes": 128849018880,
 *    "cacheBytes": 107374182400, "maxBatch": 64, "batching": true,
 *    "planStreams": 2, "cudaGraphs": true, "admissionTimeoutMs": 120000}
 * Requests (JSON):
 *   {"kind": "plan", "plan": <a plan as for gfpdb_execute_plan>}
 *   {"kind": "star", "batch": <gfpdb_star_batch spec without "queries">,
 *    "ranges": [[lo, hi], ...one per dimension]}
 * Star requests with the same "batch" text are batched: when a worker frees
 * up it takes the oldest request and every queued star request of the same
 * batch (up to maxBatch) into one run; each request's result is exactly its
 * own rows (group columns, then aggregates). Plan requests run one per
 * worker, concurrently across workers. A request starts when its
 * working-memory estimate fits hbmBudgetBytes - cacheBytes next to the
 * requests already running (one request alone always starts). */
typedef struct gfpdb_server gfpdb_server;

typedef struct gfpdb_request_stats {
  int32_t status;        /* GFPDB_OK or the request's error code */
  int32_t batch_size;    /* requests that shared this request's launches */
  int64_t submit_ns;     /* steady clock: submitted, started, finished */
  int64_t start_ns;
  int64_t end_ns;
  int64_t kernel_launches;
  int64_t cache_misses;  /* columns this request loaded into HBM */
  int32_t worker;
  int32_t pad;
} gfpdb_request_stats;

typedef struct gfpdb_server_stats {
  int64_t submitted, completed, failed;
  int64_t batches, batched_requests;
  int64_t cache_hits, cache_misses, cache_evictions;
  int64_t cache_bytes, cache_capacity, reserved_bytes, hbm_budget;
  int64_t admission_waits;
} gfpdb_server_stats;

int32_t gfpdb_server_create(const char* config_json, gfpdb_server** out);
/* Register a table held in host memory (ARROW_DEVICE_CPU or
 * ARROW_DEVICE_CUDA_HOST); its buffers must stay valid until the server is
 * destroyed. Columns are copied to HBM on first use. */
int32_t gfpdb_server_register_table(gfpdb_server* server, const char* name, const struct ArrowSchema* schema,
                                    const struct ArrowDeviceArray* array);
int32_t gfpdb_server_submit(gfpdb_server* server, const char* request_json, uint64_t* ticket);
/* Waits for a request (timeout_ms < 0: no limit; GFPDB_ETIMEDOUT when it is
 * not finished in time). On success the result is a host array the caller
 * releases (out_schema / out may be NULL to drop it); a failed request returns
 * its error. A ticket can be collected once. */
int32_t gfpdb_server_wait(gfpdb_server* server, uint64_t ticket, int64_t timeout_ms, struct ArrowSchema* out_schema,
                          struct ArrowDeviceArray* out, gfpdb_request_stats* stats);
int32_t gfpdb_server_get_stats(gfpdb_server* server, gfpdb_server_stats* out);
/* Finishes the queued requests, then frees the server. */
int32_t gfpdb_server_destroy(gfpdb_server* server);

#ifdef __cplusplus
}
#endif

#endif /* GFPDB_H */
