// Library-level C ABI: version, status strings, per-thread last-error text.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <atomic>
#include <mutex>
#include <algorithm>
#include <cstring>
#include <thread>
#include <vector>
#include "lapy_gb300.h"

static thread_local char g_last_error[512] = {0};

void lapy_set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
  snprintf(g_last_error, sizeof(g_last_error), "CUDA error %d (%s) in %s at %s:%d", (int)e,
           cudaGetErrorString(e), what, file, line);
}

void lapy_set_last_message(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

int lapy_num_sms() {
  static std::mutex mu;
  static std::vector<int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  std::lock_guard<std::mutex> lock(mu);
  if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
  if (cache[dev] == 0) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
      sms = 1;
    cache[dev] = sms;
  }
  return cache[dev];
}

static std::atomic<long long> g_launches{0};
static std::mutex g_prof_mu;
static bool g_prof_on = false;
// pcg_ms, pcg_solves, pcg_iters, rows, nnz, bytes (algorithmic),
// Lanczos (segment, block step) pairs, of which with a second CGS pass,
// then the PCG's per-phase milliseconds (kPcgPhases slots)
constexpr int kPcgPhases = LAPY_PCG_PHASES;
constexpr int kProfSlots = 8 + kPcgPhases;
static double g_prof[kProfSlots] = {0};

void lapy_count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
bool lapy_profile_enabled() { return g_prof_on; }

void lapy_profile_add_pcg(double ms, long long iters, long long rows, long long nnz, int p, int eb, int precond,
                          double coarse_bytes, bool restrict_fused) {
  std::lock_guard<std::mutex> lock(g_prof_mu);
  g_prof[0] += ms;
  g_prof[1] += 1;
  g_prof[2] += (double)iters;
  g_prof[3] += (double)rows;
  g_prof[4] += (double)nnz;
  // algorithmic bytes of the PCG iterations over the rows they touched:
  // matrix (value + column index per nonzero); Jacobi: a row pointer per
  // row, 11 vector streams of p values and 2 of the Jacobi diagonal;
  // two-level (precond 2): 12 vector streams (SpMM: P in, Q out; update: X,
  // P, Q, R in, X, R out; restriction: R in; direction: R, P in, P out), 2 of
  // the diagonal, the aggregate index per row, and the BF16 coarse inverse
  // the coarse solves streamed.  With the restriction fused into the update
  // (aggregates are row ranges) it reads no R of its own: 11 vector streams
  // and the aggregate index twice (update, direction).
  if (precond == 2 && restrict_fused)
    g_prof[5] += (double)nnz * (eb + 4) + (double)rows * (11.0 * p * eb + 2.0 * eb + 8.0) + coarse_bytes;
  else if (precond == 2)
    g_prof[5] += (double)nnz * (eb + 4) + (double)rows * (12.0 * p * eb + 2.0 * eb + 4.0) + coarse_bytes;
  else
    g_prof[5] += (double)nnz * (eb + 4) + (double)rows * (4 + 11.0 * p * eb + 2.0 * eb);
}

void lapy_profile_add_phases(const double* ms) {
  std::lock_guard<std::mutex> lock(g_prof_mu);
  for (int k = 0; k < kPcgPhases; ++k) g_prof[8 + k] += ms[k];
}

void lapy_profile_add_reorth(long long steps, long long second_passes) {
  std::lock_guard<std::mutex> lock(g_prof_mu);
  g_prof[6] += (double)steps;
  g_prof[7] += (double)second_passes;
}

extern "C" long long lapy_launch_count(void) { return g_launches.load(); }

extern "C" void lapy_profile_enable(int on) {
  std::lock_guard<std::mutex> lock(g_prof_mu);
  g_prof_on = on != 0;
}

extern "C" void lapy_profile_reset(void) {
  std::lock_guard<std::mutex> lock(g_prof_mu);
  for (double& x : g_prof) x = 0;
}

extern "C" int lapy_profile_read(double* out, int n) {
  std::lock_guard<std::mutex> lock(g_prof_mu);
  for (int i = 0; i < n && i < kProfSlots; ++i) out[i] = g_prof[i];
  return 0;
}

extern "C" int lapy_version(void) { return 10000; }

extern "C" const char* lapy_status_string(int status) {
  switch (status) {
    case LAPY_OK: return "ok";
    case LAPY_ERR_INVALID: return "invalid argument";
    case LAPY_ERR_CUDA: return "CUDA error";
    case LAPY_ERR_NOCONV: return "no convergence within the iteration cap";
    case LAPY_ERR_BREAKDOWN: return "Krylov breakdown";
    case LAPY_ERR_NAN: return "NaN or Inf in the iteration";
    case LAPY_ERR_TIMEOUT: return "bounded device-side wait timed out";
    case LAPY_ERR_WORKSPACE: return "workspace too small";
    case LAPY_ERR_PATTERN: return "matrix pattern not contained in the stiffness pattern";
    default: return "unknown status";
  }
}

extern "C" const char* lapy_last_error(void) { return g_last_error; }

// Host buffers copied back to back into one device buffer (one
// cudaMemcpyAsync per buffer, in order).
extern "C" int lapy_h2d_concat(int count, const void* const* src, const size_t* bytes, void* dst, void* pinned,
                               size_t pinned_bytes, void* stream) {
  if (count < 0 || (count > 0 && (!src || !bytes || !dst))) return LAPY_ERR_INVALID;
  size_t total = 0;
  for (int i = 0; i < count; ++i) {
    if (bytes[i] != 0 && !src[i]) return LAPY_ERR_INVALID;
    total += bytes[i];
  }
  if (total == 0) return LAPY_OK;
  if (pinned && pinned_bytes >= total) {
    // gather into the pinned buffer on a few host threads (contiguous runs
    // of buffers of about equal size), then one copy
    std::vector<size_t> off(count + 1, 0);
    for (int i = 0; i < count; ++i) off[i + 1] = off[i] + bytes[i];
    const int nthr = (int)std::max<size_t>(1, std::min<size_t>({8, (size_t)std::max(1u, std::thread::hardware_concurrency()),
                                                                  total / (4u << 20) + 1}));
    auto work = [&](int t) {
      const size_t lo = total * t / nthr, hi = total * (t + 1) / nthr;
      for (int i = 0; i < count; ++i) {
        const size_t a = std::max(lo, off[i]), b = std::min(hi, off[i + 1]);
        if (a < b) std::memcpy((char*)pinned + a, (const char*)src[i] + (a - off[i]), b - a);
      }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nthr; ++t) pool.emplace_back(work, t);
    work(0);
    for (auto& th : pool) th.join();
    const cudaError_t e = cudaMemcpyAsync(dst, pinned, total, cudaMemcpyHostToDevice, (cudaStream_t)stream);
    if (e != cudaSuccess) {
      lapy_set_last_cuda_error(e, "cudaMemcpyAsync", __FILE__, __LINE__);
      return LAPY_ERR_CUDA;
    }
    return LAPY_OK;
  }
  size_t o = 0;
  for (int i = 0; i < count; ++i) {
    if (bytes[i] == 0) continue;
    const cudaError_t e = cudaMemcpyAsync((char*)dst + o, src[i], bytes[i], cudaMemcpyHostToDevice,
                                          (cudaStream_t)stream);
    if (e != cudaSuccess) {
      lapy_set_last_cuda_error(e, "cudaMemcpyAsync", __FILE__, __LINE__);
      return LAPY_ERR_CUDA;
    }
    o += bytes[i];
  }
  return LAPY_OK;
}
