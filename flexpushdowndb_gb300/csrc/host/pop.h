// Physical operators: the GPU-backed drop-ins for the reference's
// fpdb::executor::physical operators.
//
// The interface mirrors the reference's operator contract
// (fpdb-executor/include/fpdb/executor/physical/PhysicalOp.h:41-84,
// .../physical/POpContext.h:35-40, .../message/MessageType.h:10-35):
//   - an operator is driven only through onReceive(const Envelope&),
//     clear() and getTypeString();
//   - it sees START, TUPLESET, BLOOM_FILTER and COMPLETE messages;
//   - it emits through ctx()->tell(msg), ctx()->notifyComplete() and
//     ctx()->notifyError(msg);
//   - it acts on completion when
//     ctx()->operatorMap().allComplete(POpRelationshipType::Producer) holds
//     (fpdb-executor/src/physical/LocalPOpDirectory.cpp:52-58).
// TupleSets are shared, never mutated after they are sent.
//
// The CAF actor runtime (one actor per operator, serial mailboxes,
// fpdb-executor/src/physical/POpActor.cpp:25-135) is replaced by one host
// thread delivering messages in FIFO order while every operator enqueues its
// device work on its own CUDA stream. Operators on independent branches of
// the plan (the dimension pipelines of a star query) get different streams,
// so their kernels run concurrently; a message carries an event recorded on
// its sender's stream, which the receiver's stream waits for. Under graph
// capture the streams fork from and join back to the caller's stream, so the
// captured graph has the plan's branches as parallel branches.
#pragma once

#include <deque>
#include <map>
#include <memory>
#include <optional>
#include <set>
#include <string>
#include <vector>

#include "../kernels/launch.h"
#include "expr.h"
#include "json.h"
#include "tupleset.h"

namespace gfpdb::pop {

enum class MessageType { START, TUPLESET, BLOOM_FILTER, COMPLETE, ERROR };
const char* message_type_name(MessageType t);

struct Message {
  MessageType type = MessageType::START;
  std::string sender;
  TupleSetPtr tuples;   // TUPLESET
  BloomPtr bloom;       // BLOOM_FILTER
  std::string origin;   // BLOOM_FILTER: the creator the filter belongs to, when not the sender (fused creators)
  std::string error;    // ERROR
  cudaEvent_t ready = nullptr;  // recorded on the sender's stream after its work for this message
  int stream = 0;               // the sender's stream index
};

// The reference wraps a message in an Envelope; here the envelope is the
// message itself plus its receiver.
struct Envelope {
  Message message;
  const Message& getMessage() const { return message; }
};

enum class POpRelationshipType { Producer, Consumer };

class LocalPOpDirectory {
 public:
  void add(const std::string& name, POpRelationshipType rel);
  void setComplete(const std::string& name);
  bool isComplete(const std::string& name) const;
  bool allComplete(POpRelationshipType rel) const;
  bool has(const std::string& name, POpRelationshipType rel) const;
  std::vector<std::string> names(POpRelationshipType rel) const;

 private:
  struct Entry {
    std::set<POpRelationshipType> rels;
    bool complete = false;
  };
  std::map<std::string, Entry> entries_;
};

class Execution;
class PhysicalOp;

// Streams a plan runs on unless its "streams" option says otherwise.
constexpr int kDefaultPlanStreams = 4;

class POpContext {
 public:
  POpContext(Execution* exec, PhysicalOp* op) : exec_(exec), op_(op) {}
  // Send to every consumer, or to the named ones.
  void tell(Message msg);
  void tell(Message msg, const std::vector<std::string>& consumers);
  void notifyComplete();
  void notifyError(const std::string& error);
  LocalPOpDirectory& operatorMap();
  cudaStream_t stream() const;
  // Another stream of the execution (the k-th after this operator's, round
  // robin; the operator's own when the plan runs on one stream), for work an
  // operator runs beside its own.
  cudaStream_t sideStream(int k) const;
  // Makes `waiter` wait for the work issued so far on `on` (an event).
  void streamWait(cudaStream_t waiter, cudaStream_t on);
  bool isComplete() const { return complete_; }

 private:
  Execution* exec_;
  PhysicalOp* op_;
  bool complete_ = false;
};

class PhysicalOp {
 public:
  PhysicalOp(std::string name, std::string type) : name_(std::move(name)), type_(std::move(type)) {}
  virtual ~PhysicalOp() = default;

  virtual void onReceive(const Envelope& msg) = 0;
  virtual void clear() {}
  virtual std::string getTypeString() const { return type_; }

  const std::string& name() const { return name_; }
  std::vector<std::string>& producers() { return producers_; }
  std::vector<std::string>& consumers() { return consumers_; }
  void setProjectColumnNames(std::vector<std::string> c) { projectColumnNames_ = std::move(c); }
  const std::vector<std::string>& getProjectColumnNames() const { return projectColumnNames_; }

  POpContext* ctx() { return ctx_.get(); }
  void setContext(std::unique_ptr<POpContext> c) { ctx_ = std::move(c); }
  LocalPOpDirectory& directory() { return directory_; }

 protected:
  std::string name_;
  std::string type_;
  std::vector<std::string> producers_;
  std::vector<std::string> consumers_;
  std::vector<std::string> projectColumnNames_;
  std::unique_ptr<POpContext> ctx_;
  LocalPOpDirectory directory_;
};

// Input tables of a plan, by name.
struct InputTable {
  TupleSetPtr device;                 // already resident
  const ArrowSchema* schema = nullptr;  // or imported at scan time
  const ArrowDeviceArray* array = nullptr;
};

struct ExecStats {
  int64_t kernel_launches = 0;
  int64_t h2d_bytes = 0;
  int64_t d2h_bytes = 0;
  int64_t messages = 0;
  int64_t num_ops = 0;
};

// Thrown by Execution::execute when a deferred output overflowed the
// capacity it was given (a join whose build keys repeat): the caller runs the
// plan again with exact sizes.
struct NeedsExactSizes : std::exception {
  const char* what() const noexcept override { return "deferred output overflowed its capacity"; }
};

class Execution {
 public:
  Execution(cudaStream_t stream) : stream_(stream) {}

  // Deferred sizes (default): operators chain on the stream without waiting
  // for row counts; the plan synchronizes once at the end.
  void setDeferred(bool on) { deferred_ = on; }
  // Capture mode: execute() only enqueues (no final synchronization) and
  // hands the status checks to the caller, which runs them after each
  // replay of the captured graph.
  void setCapturing(bool on) { capturing_ = on; }
  std::vector<DeferredCheck> takeCapturedChecks() { return std::move(captured_checks_); }

  void add(std::unique_ptr<PhysicalOp> op);
  PhysicalOp* op(const std::string& name);
  void connect();  // fill producers from consumers and each op's directory
  void setInputs(std::map<std::string, InputTable> inputs) { inputs_ = std::move(inputs); }
  const InputTable& input(const std::string& name) const;

  // START every operator, deliver messages until all are complete, return
  // the CollatePOp's TupleSet (Execution::execute, fpdb-executor/src/Execution.cpp:44-50).
  TupleSetPtr execute();

  void post(const std::string& to, Message msg);
  void markComplete(const std::string& name);
  void error(const std::string& from, const std::string& msg);
  cudaStream_t stream() const { return stream_; }
  ExecStats stats() const { return stats_; }

  // Up to n streams (the caller's plus n - 1 of this thread's pool); 1 runs
  // every operator on the caller's stream. Call before execute().
  void setStreams(int n) { n_streams_ = n < 1 ? 1 : n; }
  int streamCount() const { return static_cast<int>(streams_.size()); }
  cudaStream_t streamOf(const PhysicalOp* op) const;
  cudaStream_t sideStreamOf(const PhysicalOp* op, int k) const;
  void streamWait(cudaStream_t waiter, cudaStream_t on);
  // Stamps an outgoing message with its sender's stream and ready event.
  void stamp(Message& msg, const PhysicalOp* sender);
  ~Execution();

 private:
  void assignStreams();
  cudaStream_t stream_;
  int n_streams_ = 1;
  std::vector<cudaStream_t> streams_;           // [0] is the caller's stream
  std::map<const PhysicalOp*, int> op_stream_;
  size_t events_used_ = 0;  // of this thread's event pool, in this execution
  std::vector<TupleSetPtr> retained_tuples_;   // message payloads, kept until the plan has finished
  std::vector<BloomPtr> retained_blooms_;
  std::vector<std::unique_ptr<PhysicalOp>> ops_;
  std::map<std::string, PhysicalOp*> by_name_;
  std::deque<std::pair<std::string, Message>> mailbox_;
  std::map<std::string, InputTable> inputs_;
  std::string error_;
  ExecStats stats_;
  bool deferred_ = true;
  bool capturing_ = false;
  std::vector<DeferredCheck> captured_checks_;
};

// Join tables and probes on one or several key columns (the C ABI's hash
// join and HashJoinArrowPOp share them).
// With `mark` the table keeps a matched flag per build row (outer and semi
// joins).
// `filters` are bloom filters the build side's rows must pass (a bloom
// selection folded into the build): tested in the table build when they are
// all on the single integer key column and the join keeps no unmatched build
// rows (no `mark`), otherwise applied by a selection before it.
JoinTable build_join_table(const TupleSetPtr& build, const std::vector<std::string>& keys, double load_factor,
                           cudaStream_t s, bool mark = false, const std::vector<BloomProbe>& filters = {});
// The build side with `filters` applied: unchanged with the filters moved
// into *in_build when every one is on `key` (an int32, int64 or date32
// column; empty `key`: never) and there are at most kJoinBuildFiltersMax,
// else the rows that pass them all.
TupleSetPtr filter_build_side(const TupleSetPtr& build, const std::string& key, const std::vector<BloomProbe>& filters,
                              cudaStream_t s, std::vector<BloomPtr>* in_build);
TupleSetPtr join_probe_keys(const std::string& join_name, const JoinTable& table, const std::vector<std::string>& proj,
                            const std::vector<std::string>& probe_keys, const TupleSetPtr& ts, cudaStream_t s);

// The reference's JoinType (fpdb-plan/include/fpdb/plan/prephysical/JoinType.h:13-20),
// the values of GFPDB_JOIN_*. LEFT keeps every build row (HashJoinArrowKernel
// hands Arrow the build side as its right input and asks for RIGHT_OUTER),
// RIGHT every probe row; LEFT_SEMI emits the build rows with a match,
// RIGHT_SEMI the probe rows with a match, each with that side's columns only
// (HashJoinArrowKernel.cpp:164-195).
enum class JoinKind { Inner = 0, Left = 1, Right = 2, Full = 3, LeftSemi = 4, RightSemi = 5 };
JoinKind join_kind_from_name(const std::string& name);
bool join_kind_marks(JoinKind k);  // the table keeps build-row matched flags
// One probe batch's output rows (null for LEFT_SEMI, whose rows come at the
// end); non-inner joins take one integer key column per side.
TupleSetPtr join_probe_kind(const std::string& join_name, JoinKind kind, const JoinTable& table,
                            const std::vector<std::string>& proj, const std::vector<std::string>& probe_keys,
                            const TupleSetPtr& ts, cudaStream_t s);
// The rows emitted once every probe batch is in: the unmatched build rows
// with null probe columns (LEFT, FULL), the matched build rows (LEFT_SEMI);
// null for the other kinds. probe_fields: the probe side's schema.
TupleSetPtr join_finish_kind(const std::string& join_name, JoinKind kind, const JoinTable& table,
                             const std::vector<Field>& probe_fields, const std::vector<std::string>& proj,
                             cudaStream_t s);

// A file of the local file system, whole (the scan operators' input).
std::vector<uint8_t> read_local_file(const std::string& path);

// Aggregate functions of a group-by spec: [{"function", "name", "expr"}],
// functions SUM, COUNT (without expr: count of rows), MIN, MAX, AVG and
// AVG_REDUCE (no expr; the second phase of a parallel AVG).
std::vector<GroupAggregate> parse_aggregates(const json::Value& list);

// The bloom-filter operators of a join graph's predicate transfer, as JSON
// (format documented with gfpdb_plan_predicate_transfer in include/gfpdb.h).
std::string plan_predicate_transfer(const json::Value& spec);

// Build an Execution from a JSON plan (format documented with
// gfpdb_execute_plan in include/gfpdb.h).
std::unique_ptr<Execution> build_execution(const json::Value& plan, cudaStream_t stream);
// The plan after pipeline fusion (what build_execution runs when
// "fusePipelines" is true, the default): bloom selections chained on one
// input merged, bloom selections feeding only an inner join's build side
// folded into the join build, chains of inner joins merged.
json::Value fuse_pipelines(const json::Value& plan);
void validate_plan(const json::Value& plan);

}  // namespace gfpdb::pop
