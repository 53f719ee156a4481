// Host runtime: errors, CUDA checks, device buffers, launch accounting.
//
// The reference reports failures as tl::expected<T, std::string> and turns
// them into ErrorMessages (fpdb-executor/src/physical/POpContext.cpp:190-195).
// Inside this library a failure is a gfpdb::Error exception carrying one of
// the GFPDB_E* codes; the C-ABI layer converts it to a status code plus a
// thread-local message.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../../include/gfpdb.h"

namespace gfpdb {

class Error : public std::runtime_error {
 public:
  Error(int32_t code, const std::string& msg) : std::runtime_error(msg), code_(code) {}
  int32_t code() const { return code_; }

 private:
  int32_t code_;
};

[[noreturn]] void fail(int32_t code, const std::string& msg);

// Message of the last failed C-ABI call on this thread.
std::string& last_error();

// Run `f` for a C entry point: GFPDB_OK, or the failure's code with its
// message stored in last_error().
template <typename F>
int32_t guarded(F&& f) {
  try {
    last_error().clear();
    f();
    return GFPDB_OK;
  } catch (const Error& e) {
    last_error() = e.what();
    return e.code();
  } catch (const std::bad_alloc&) {
    last_error() = "host allocation failed";
    return GFPDB_ENOMEM;
  } catch (const std::exception& e) {
    last_error() = e.what();
    return GFPDB_EINVAL;
  }
}
void check_cuda(cudaError_t e, const char* what);
#define GF_CUDA(call) ::gfpdb::check_cuda((call), #call)

// Every kernel launch in the library goes through this counter so a caller
// can tell how many device kernels a call issued.
extern std::atomic<uint64_t> g_kernel_launches;
// Kernel launches of the calling thread (what one request of a worker
// thread launched, when several threads share the GPU).
uint64_t& thread_kernel_launches();
inline void count_launch(uint64_t n = 1) {
  g_kernel_launches.fetch_add(n, std::memory_order_relaxed);
  thread_kernel_launches() += n;
}
// Checks the launch that was just issued and counts it.
void after_launch(const char* kernel_name);

// Per-thread byte counters of host<->device copies, read by plan execution.
struct CopyCounters {
  int64_t h2d = 0;
  int64_t d2h = 0;
  int64_t in_place = 0;  // bytes of page-locked host columns kernels read in place (the columns' size)
};
CopyCounters& copy_counters();

int current_device();
void ensure_device();            // gfpdb_device_init on first use
int num_sms();                   // SM count of the current device
int max_smem_optin();            // opt-in shared memory per block

// Stream-ordered device allocation. Memory comes from the device's default
// memory pool with an unbounded release threshold, so repeated queries reuse
// pages instead of returning them to the driver.
class DeviceBuffer {
 public:
  DeviceBuffer(int64_t bytes, cudaStream_t stream);
  // Borrowed memory: never freed by this object.
  DeviceBuffer(void* borrowed, int64_t bytes) : ptr_(borrowed), bytes_(bytes), owned_(false) {}
  ~DeviceBuffer();
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;

  void* data() const { return ptr_; }
  int64_t size() const { return bytes_; }
  template <typename T>
  T* as() const {
    return static_cast<T*>(ptr_);
  }

 private:
  void* ptr_ = nullptr;
  int64_t bytes_ = 0;
  bool owned_ = true;
  cudaStream_t stream_ = nullptr;
};
using BufferPtr = std::shared_ptr<DeviceBuffer>;

inline BufferPtr make_buffer(int64_t bytes, cudaStream_t stream) {
  return std::make_shared<DeviceBuffer>(bytes, stream);
}

// A bump arena over one device allocation. While an arena is active on a
// thread, every DeviceBuffer that thread creates is carved from it and is
// never freed on its own: the arena's memory is reused as a whole. Used to
// capture a plan into a CUDA graph, whose kernels then see fixed addresses.
class Arena {
 public:
  Arena(int64_t bytes, cudaStream_t s);
  void* take(int64_t bytes);  // 256-byte aligned; throws GFPDB_ENOMEM when full
  int64_t used() const { return used_; }
  int64_t size() const { return size_; }
  void reset() { used_ = 0; }

 private:
  BufferPtr base_;
  int64_t size_ = 0;
  int64_t used_ = 0;
};
// Activate `a` for this thread (nullptr deactivates).
void set_thread_arena(Arena* a);

// Buffers that must start out filled with one byte value, 0 or 0xFF (status
// blocks, tickets, tile states, hash-table slots, filter words). Normally an
// allocation and a memset on the stream. While a fill pool is active on the
// thread (a plan being captured into a CUDA graph) they are carved from the
// pool's region for that value and size class, which the graph fills with one
// memset at its start, so the plan's operators add no memset nodes of their
// own. Small buffers come from regions filled on the capturing stream before
// anything else; large ones (capacity-sized tables and filters) from regions
// filled on a side stream, overlapping the plan's first operators, and a
// stream that takes one waits for that fill.
BufferPtr make_filled(int64_t bytes, int value, cudaStream_t s);

constexpr int64_t kFillLargeBytes = 64 * 1024;

struct FillPool {
  char* base[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [small, large][zeros, 0xFF]
  int64_t size[2][2] = {{0, 0}, {0, 0}};
  int64_t used[2][2] = {{0, 0}, {0, 0}};
  cudaEvent_t large_ready = nullptr;  // recorded after the large regions are filled
};
// Activate `p` for this thread (nullptr deactivates).
void set_thread_fill_pool(FillPool* p);
// Bytes this thread has asked make_filled for, per size class and value
// ([small, large][zeros, 0xFF]), each request rounded up to 256.
void thread_filled_bytes(int64_t out[2][2]);
// Bytes this thread has allocated through DeviceBuffer (rounded to 256).
int64_t thread_alloc_bytes();

void memcpy_h2d(void* dst, const void* src, int64_t n, cudaStream_t s);
void memcpy_d2h(void* dst, const void* src, int64_t n, cudaStream_t s);
void sync(cudaStream_t s);

// Per-call status block that every kernel of one operator call shares: a
// device error word (first error code + detail) and counters, zeroed by a
// single memset. Read back with read_status() after the call's kernels.
struct DevStatus {
  int32_t code;     // 0 = ok, else a GFPDB_E* code raised on the device
  int32_t detail;   // kernel-specific detail (e.g. which wait gave up)
  int64_t value;    // kernel-specific (e.g. rows produced)
  int64_t aux[6];
};
static_assert(sizeof(DevStatus) == 64, "status block is one 64-byte line");

void raise_device_status(const DevStatus& st, const char* where);

// Deferred sizes. While a plan runs in deferred mode, operators do not wait
// for their kernels: outputs are allocated at an upper bound and carry their
// true row count in device memory, and each call's status block is recorded
// here instead of being read back. The plan executor synchronizes once at the
// end and checks them all. A record with `capacity` > 0 also checks that the
// count its kernel produced (DevStatus::value) fit the allocated capacity;
// a miss means the plan must be re-run with exact sizes.
struct DeferredCheck {
  BufferPtr owner;
  const DevStatus* status;
  const char* where;
  int64_t capacity;
};
bool deferred_mode();
void set_deferred_mode(bool on);
// How scans bring host inputs to the device: 0 = copy engine, 1 = SM loads,
// 2 = no copy (kernels read page-locked host columns directly).
int host_copy_mode();
void set_host_copy_mode(int mode);
void defer_check(BufferPtr owner, const DevStatus* status, const char* where, int64_t capacity = 0);
// Reads every recorded status (the stream must be synchronized). Raises the
// first device error; returns false if some output overflowed its capacity.
bool run_deferred_checks(cudaStream_t s);
void clear_deferred_checks();
// Move the recorded checks out (a captured plan keeps them for its replays),
// and run a kept list (the stream must be synchronized).
std::vector<DeferredCheck> take_deferred_checks();
bool run_checks(const std::vector<DeferredCheck>& checks, cudaStream_t s);

// Device row count of a TupleSet-like input: min(*n_dev, capacity) or capacity.
__host__ __device__ inline int64_t clamp_rows(const int64_t* n_dev, int64_t capacity) {
  if (n_dev == nullptr) return capacity;
  const int64_t n = *n_dev;
  return n < capacity ? (n < 0 ? 0 : n) : capacity;
}

// Optional per-launch timing (gfpdb_profile_*): events on the launching
// stream around one kernel plus its algorithmic bytes.
class ProfScope {
 public:
  ProfScope(const char* name, cudaStream_t s);
  // Record the stop event; bytes may be refined later with set_bytes().
  void stop(double bytes);
  void set_bytes(double bytes);
  // Bytes = per_in * rows_in + per_out * rows_out, with either row count
  // read from device memory when the profile is read (deferred sizes).
  void set_bytes_model(const int64_t* rows_in_dev, int64_t rows_in, double per_in, const int64_t* rows_out_dev,
                       double per_out, std::shared_ptr<class DeviceBuffer> keep,
                       std::shared_ptr<class DeviceBuffer> keep2 = nullptr);

 private:
  int64_t index_ = -1;
  cudaStream_t stream_;
};
void prof_enable(bool on);
void prof_reset();
void prof_read(const std::string& name, int64_t* launches, double* ms, double* bytes);
std::string prof_kernels();

}  // namespace gfpdb
