#include "runtime.h"

#include <mutex>
#include <vector>

namespace gfpdb {

std::atomic<uint64_t> g_kernel_launches{0};

uint64_t& thread_kernel_launches() {
  thread_local uint64_t n = 0;
  return n;
}

void fail(int32_t code, const std::string& msg) { throw Error(code, msg); }

std::string& last_error() {
  thread_local std::string msg;
  return msg;
}

void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    fail(e == cudaErrorMemoryAllocation ? GFPDB_ENOMEM : GFPDB_ECUDA,
         std::string("CUDA error in ") + what + ": " + cudaGetErrorName(e) + " (" +
             cudaGetErrorString(e) + ")");
  }
}

void after_launch(const char* kernel_name) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    fail(GFPDB_ECUDA, std::string("launch of ") + kernel_name + " failed: " + cudaGetErrorName(e) +
                          " (" + cudaGetErrorString(e) + ")");
  }
  count_launch();
}

CopyCounters& copy_counters() {
  thread_local CopyCounters c;
  return c;
}

namespace {
struct DeviceInfo {
  bool ready = false;
  int sms = 0;
  int smem_optin = 0;
};
std::mutex g_dev_mu;
std::vector<DeviceInfo> g_devs;
}  // namespace

int current_device() {
  int d = 0;
  GF_CUDA(cudaGetDevice(&d));
  return d;
}

static DeviceInfo& info_for(int dev) {
  std::lock_guard<std::mutex> lk(g_dev_mu);
  if (g_devs.empty()) {
    int n = 0;
    GF_CUDA(cudaGetDeviceCount(&n));
    if (n <= 0) fail(GFPDB_ECUDA, "no CUDA device is visible");
    g_devs.resize(n);
  }
  if (dev < 0 || dev >= static_cast<int>(g_devs.size())) fail(GFPDB_EINVAL, "device index out of range");
  DeviceInfo& di = g_devs[dev];
  if (!di.ready) {
    cudaDeviceProp prop;
    GF_CUDA(cudaGetDeviceProperties(&prop, dev));
    if (prop.major < 10) {
      fail(GFPDB_EUNSUPPORTED, std::string("device ") + prop.name + " is not a Blackwell (sm_10x) GPU");
    }
    di.sms = prop.multiProcessorCount;
    di.smem_optin = static_cast<int>(prop.sharedMemPerBlockOptin);
    cudaMemPool_t pool;
    GF_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
    uint64_t threshold = UINT64_MAX;
    GF_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold));
    di.ready = true;
  }
  return di;
}

void ensure_device() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) check_cuda(e, "cudaGetDevice");
  info_for(dev);
}

int num_sms() { return info_for(current_device()).sms; }
int max_smem_optin() { return info_for(current_device()).smem_optin; }

namespace {
thread_local Arena* g_thread_arena = nullptr;
thread_local int64_t g_thread_alloc = 0;
}  // namespace

void set_thread_arena(Arena* a) { g_thread_arena = a; }
int64_t thread_alloc_bytes() { return g_thread_alloc; }

namespace {
thread_local FillPool* g_fill_pool = nullptr;
thread_local int64_t g_filled[2][2] = {{0, 0}, {0, 0}};
}  // namespace

void set_thread_fill_pool(FillPool* p) { g_fill_pool = p; }

void thread_filled_bytes(int64_t out[2][2]) {
  for (int t = 0; t < 2; ++t)
    for (int k = 0; k < 2; ++k) out[t][k] = g_filled[t][k];
}

BufferPtr make_filled(int64_t bytes, int value, cudaStream_t s) {
  if (value != 0 && value != 0xFF) fail(GFPDB_EINVAL, "make_filled takes the byte values 0 and 0xFF");
  const int k = value == 0 ? 0 : 1;
  const int t = bytes >= kFillLargeBytes ? 1 : 0;
  const int64_t n = ((bytes > 16 ? bytes : 16) + 255) / 256 * 256;
  g_filled[t][k] += n;
  FillPool* fp = g_fill_pool;
  if (fp != nullptr && fp->used[t][k] + n <= fp->size[t][k]) {
    char* p = fp->base[t][k] + fp->used[t][k];
    fp->used[t][k] += n;
    if (t == 1) GF_CUDA(cudaStreamWaitEvent(s, fp->large_ready, 0));
    return std::make_shared<DeviceBuffer>(p, bytes);
  }
  auto b = make_buffer(bytes, s);
  if (bytes > 0) GF_CUDA(cudaMemsetAsync(b->data(), value, static_cast<size_t>(bytes), s));
  return b;
}

Arena::Arena(int64_t bytes, cudaStream_t s) : size_(bytes) {
  Arena* saved = g_thread_arena;
  g_thread_arena = nullptr;  // the arena's own memory comes from the pool
  base_ = make_buffer(bytes, s);
  g_thread_arena = saved;
}

void* Arena::take(int64_t bytes) {
  const int64_t n = (bytes + 255) / 256 * 256;
  if (used_ + n > size_) fail(GFPDB_ENOMEM, "plan arena exhausted");
  void* p = base_->as<char>() + used_;
  used_ += n;
  return p;
}

DeviceBuffer::DeviceBuffer(int64_t bytes, cudaStream_t stream) : bytes_(bytes), owned_(true), stream_(stream) {
  if (bytes < 0) fail(GFPDB_EINVAL, "negative allocation size");
  // Zero-byte buffers still get a distinct valid pointer so Arrow consumers
  // never see NULL data buffers for empty columns.
  int64_t n = bytes > 0 ? bytes : 16;
  g_thread_alloc += (n + 255) / 256 * 256;
  if (g_thread_arena != nullptr) {
    ptr_ = g_thread_arena->take(n);
    owned_ = false;
    return;
  }
  GF_CUDA(cudaMallocAsync(&ptr_, static_cast<size_t>(n), stream));
}

DeviceBuffer::~DeviceBuffer() {
  if (owned_ && ptr_ != nullptr) {
    // Errors are swallowed: destructors must not throw, and a failing free
    // means the context is already gone.
    (void)cudaFreeAsync(ptr_, stream_);
  }
}

void memcpy_h2d(void* dst, const void* src, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  GF_CUDA(cudaMemcpyAsync(dst, src, static_cast<size_t>(n), cudaMemcpyHostToDevice, s));
  copy_counters().h2d += n;
}

void memcpy_d2h(void* dst, const void* src, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  GF_CUDA(cudaMemcpyAsync(dst, src, static_cast<size_t>(n), cudaMemcpyDeviceToHost, s));
  copy_counters().d2h += n;
}

void sync(cudaStream_t s) { GF_CUDA(cudaStreamSynchronize(s)); }

namespace {
struct ProfRecord {
  std::string name;
  cudaEvent_t start = nullptr;
  cudaEvent_t stop = nullptr;
  double bytes = 0;
  // optional byte model evaluated at read time
  bool model = false;
  const int64_t* rows_in_dev = nullptr;
  int64_t rows_in = 0;
  double per_in = 0;
  const int64_t* rows_out_dev = nullptr;
  double per_out = 0;
  std::shared_ptr<DeviceBuffer> keep, keep2;
};
std::mutex g_prof_mu;
std::vector<ProfRecord> g_prof;
std::atomic<bool> g_prof_on{false};
}  // namespace

ProfScope::ProfScope(const char* name, cudaStream_t s) : stream_(s) {
  if (!g_prof_on.load(std::memory_order_relaxed)) return;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) == cudaSuccess && cap != cudaStreamCaptureStatusNone) return;
  ProfRecord r;
  r.name = name;
  GF_CUDA(cudaEventCreate(&r.start));
  GF_CUDA(cudaEventCreate(&r.stop));
  GF_CUDA(cudaEventRecord(r.start, s));
  std::lock_guard<std::mutex> lk(g_prof_mu);
  index_ = static_cast<int64_t>(g_prof.size());
  g_prof.push_back(r);
}

void ProfScope::stop(double bytes) {
  if (index_ < 0) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  GF_CUDA(cudaEventRecord(g_prof[index_].stop, stream_));
  g_prof[index_].bytes = bytes;
}

void ProfScope::set_bytes(double bytes) {
  if (index_ < 0) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof[index_].bytes = bytes;
}

void ProfScope::set_bytes_model(const int64_t* rows_in_dev, int64_t rows_in, double per_in,
                                const int64_t* rows_out_dev, double per_out, std::shared_ptr<DeviceBuffer> keep,
                                std::shared_ptr<DeviceBuffer> keep2) {
  if (index_ < 0) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  ProfRecord& r = g_prof[index_];
  r.model = true;
  r.rows_in_dev = rows_in_dev;
  r.rows_in = rows_in;
  r.per_in = per_in;
  r.rows_out_dev = rows_out_dev;
  r.per_out = per_out;
  r.keep = std::move(keep);
  r.keep2 = std::move(keep2);
}

void prof_enable(bool on) { g_prof_on.store(on); }

void prof_reset() {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  for (auto& r : g_prof) {
    if (r.start) cudaEventDestroy(r.start);
    if (r.stop) cudaEventDestroy(r.stop);
  }
  g_prof.clear();
}

void prof_read(const std::string& name, int64_t* launches, double* ms, double* bytes) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  int64_t n = 0;
  double t = 0, b = 0;
  for (auto& r : g_prof) {
    if (r.name != name) continue;
    GF_CUDA(cudaEventSynchronize(r.stop));
    float e = 0;
    GF_CUDA(cudaEventElapsedTime(&e, r.start, r.stop));
    ++n;
    t += e;
    if (r.model) {
      int64_t in = r.rows_in, out = 0;
      if (r.rows_in_dev) GF_CUDA(cudaMemcpy(&in, r.rows_in_dev, sizeof(in), cudaMemcpyDeviceToHost));
      if (r.rows_out_dev) GF_CUDA(cudaMemcpy(&out, r.rows_out_dev, sizeof(out), cudaMemcpyDeviceToHost));
      if (in > r.rows_in) in = r.rows_in;
      b += r.per_in * static_cast<double>(in) + r.per_out * static_cast<double>(out);
    } else {
      b += r.bytes;
    }
  }
  *launches = n;
  *ms = t;
  *bytes = b;
}

std::string prof_kernels() {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  std::vector<std::string> seen;
  std::string out;
  for (auto& r : g_prof) {
    bool dup = false;
    for (auto& s : seen) dup |= s == r.name;
    if (dup) continue;
    seen.push_back(r.name);
    out += r.name + "\n";
  }
  return out;
}

namespace {
thread_local bool g_deferred = false;
thread_local std::vector<DeferredCheck> g_checks;
}  // namespace

bool deferred_mode() { return g_deferred; }
void set_deferred_mode(bool on) { g_deferred = on; }

namespace {
thread_local int g_host_copy = 0;
}
int host_copy_mode() { return g_host_copy; }
void set_host_copy_mode(int mode) { g_host_copy = mode; }

void defer_check(BufferPtr owner, const DevStatus* status, const char* where, int64_t capacity) {
  g_checks.push_back(DeferredCheck{std::move(owner), status, where, capacity});
}

void clear_deferred_checks() { g_checks.clear(); }

std::vector<DeferredCheck> take_deferred_checks() {
  std::vector<DeferredCheck> out;
  out.swap(g_checks);
  return out;
}

bool run_checks(const std::vector<DeferredCheck>& checks, cudaStream_t s) {
  bool fits = true;
  std::vector<DevStatus> host(checks.size());
  for (size_t i = 0; i < checks.size(); ++i)
    GF_CUDA(cudaMemcpyAsync(&host[i], checks[i].status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
  sync(s);
  for (size_t i = 0; i < checks.size(); ++i) {
    raise_device_status(host[i], checks[i].where);
    if (checks[i].capacity > 0 && host[i].value > checks[i].capacity) fits = false;
  }
  return fits;
}

bool run_deferred_checks(cudaStream_t s) {
  auto checks = take_deferred_checks();
  return run_checks(checks, s);
}

void raise_device_status(const DevStatus& st, const char* where) {
  if (st.code == 0) return;
  std::string what;
  switch (st.code) {
    case GFPDB_ETIMEDOUT: what = "a bounded device wait gave up"; break;
    case GFPDB_EDEVICE: what = "device error"; break;
    case GFPDB_ENOMEM: what = "device table or arena full"; break;
    case GFPDB_EINVAL: what = "invalid value on device"; break;
    default: what = "device status " + std::to_string(st.code);
  }
  fail(st.code, std::string(where) + ": " + what + " (detail " + std::to_string(st.detail) + ")");
}

}  // namespace gfpdb
