// Runtime pieces of the C-ABI: error messages, launch counting, device info.
#include "jscc_common.cuh"

#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace jscc {

static thread_local char g_err[1024] = {0};

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

std::atomic<unsigned long long>& launch_counter() {
  static std::atomic<unsigned long long> c{0};
  return c;
}

int num_sms() {
  // Cached per device; the library is used from one device per process in
  // practice, but the cache is keyed by device to stay correct otherwise.
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (cache[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 148;
    cache[dev] = n;
  }
  return cache[dev];
}

// ---------------------------------------------------------------- kernel timing
struct TimedLaunch {
  const char* name;
  cudaEvent_t start, stop;
};

static std::mutex g_tmu;
static bool g_timing = false;
static std::vector<TimedLaunch> g_launches;
static std::vector<cudaEvent_t> g_event_pool;
static thread_local cudaEvent_t g_pending_start = nullptr;

static cudaEvent_t take_event() {
  if (!g_event_pool.empty()) {
    cudaEvent_t e = g_event_pool.back();
    g_event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

bool timing_enabled() { return g_timing; }

void timing_begin(cudaStream_t st) {
  std::lock_guard<std::mutex> lk(g_tmu);
  g_pending_start = take_event();
  if (g_pending_start) cudaEventRecord(g_pending_start, st);
}

void timing_end(const char* name, cudaStream_t st) {
  std::lock_guard<std::mutex> lk(g_tmu);
  cudaEvent_t stop = take_event();
  if (!g_pending_start || !stop) return;
  cudaEventRecord(stop, st);
  g_launches.push_back({name, g_pending_start, stop});
  g_pending_start = nullptr;
}

int set_bulk_poll_limit(uint32_t polls, bool reset);  // sparse_ops.cu
int set_gemm_poll_limit(uint32_t polls, bool reset);  // batched_gemm.cu
int set_sc_poll_limit(uint32_t polls, bool reset);    // sc_projector.cu

}  // namespace jscc

extern "C" {

int jscc_set_wait_limit(int64_t polls) {
  JSCC_REQUIRE(polls <= (int64_t)UINT32_MAX, "jscc_set_wait_limit: %lld polls is above 2^32 - 1", (long long)polls);
  const bool reset = polls < 0;
  const uint32_t v = reset ? 0u : (uint32_t)polls;
  int rc = jscc::set_bulk_poll_limit(v, reset);
  if (rc != JSCC_OK) return rc;
  rc = jscc::set_sc_poll_limit(v, reset);
  if (rc != JSCC_OK) return rc;
  return jscc::set_gemm_poll_limit(v, reset);
}

void jscc_kernel_timing_enable(int enable) {
  std::lock_guard<std::mutex> lk(jscc::g_tmu);
  jscc::g_timing = enable != 0;
}

int jscc_kernel_timing_collect(char* buf, size_t buf_bytes) {
  using namespace jscc;
  std::lock_guard<std::mutex> lk(g_tmu);
  std::map<std::string, std::pair<long long, double>> agg;
  for (auto& l : g_launches) {
    if (cudaEventSynchronize(l.stop) != cudaSuccess) {
      set_error("jscc_kernel_timing_collect: event sync failed");
      return JSCC_ERR_CUDA;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, l.start, l.stop);
    auto& a = agg[l.name];
    a.first += 1;
    a.second += ms;
    g_event_pool.push_back(l.start);
    g_event_pool.push_back(l.stop);
  }
  g_launches.clear();
  std::string out;
  char line[256];
  for (auto& kv : agg) {
    snprintf(line, sizeof(line), "%s %lld %.6f\n", kv.first.c_str(), kv.second.first, kv.second.second);
    out += line;
  }
  if (buf && buf_bytes > 0) {
    size_t n = out.size() < buf_bytes - 1 ? out.size() : buf_bytes - 1;
    memcpy(buf, out.data(), n);
    buf[n] = 0;
  }
  return JSCC_OK;
}


const char* jscc_last_error(void) { return jscc::g_err; }

int jscc_abi_version(void) { return 7; }

unsigned long long jscc_launch_count(void) { return jscc::launch_counter().load(); }

void jscc_reset_launch_count(void) { jscc::launch_counter().store(0); }

void jscc_count_graph_launches(unsigned long long n) { jscc::launch_counter().fetch_add(n); }

}  // extern "C"
