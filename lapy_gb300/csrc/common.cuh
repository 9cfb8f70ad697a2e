// Shared device/host helpers for the lapy_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <algorithm>
#include "lapy_gb300.h"

#define LAPY_CUDA_TRY(expr)                                   \
  do {                                                        \
    cudaError_t _e = (expr);                                  \
    if (_e != cudaSuccess) {                                  \
      lapy_set_last_cuda_error(_e, #expr, __FILE__, __LINE__); \
      return LAPY_ERR_CUDA;                                   \
    }                                                         \
  } while (0)

#define LAPY_TRY(expr)            \
  do {                            \
    int _s = (expr);              \
    if (_s != LAPY_OK) return _s; \
  } while (0)

void lapy_set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line);
void lapy_set_last_message(const char* fmt, ...);

// Launch accounting (every kernel launch site calls lapy_check_launch).
void lapy_count_launch();
// PCG profile accumulation (enabled by lapy_profile_enable).
bool lapy_profile_enabled();
void lapy_profile_add_pcg(double ms, long long iters, long long rows, long long nnz, int p, int elem_bytes,
                          int precond, double coarse_bytes, bool restrict_fused);
void lapy_profile_add_reorth(long long steps, long long second_passes);
// Per-phase device time of the persistent PCG (profile mode): the interval
// between consecutive grid-barrier exits, accumulated per phase: initialisation,
// SpMM (Q = K P), update (X, R), coarse restriction, coarse solve, direction
// update, final publication.
constexpr int kPcgPhases = LAPY_PCG_PHASES;
void lapy_profile_add_phases(const double* ms);

static inline int lapy_check_launch(const char* what) {
  lapy_count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    lapy_set_last_cuda_error(e, what, __FILE__, __LINE__);
    return LAPY_ERR_CUDA;
  }
  return LAPY_OK;
}

static inline unsigned lapy_ceil_div(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

// Number of SMs of the current device (cached per device).
int lapy_num_sms();

// ---------------------------------------------------------------------------
// Warp / block reductions (deterministic: fixed shuffle tree, fixed warp order)
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block-wide sum; every thread gets the result. `sh` must hold >= 32 T.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  T r = (threadIdx.x < nw) ? sh[threadIdx.x] : T(0);
  if (wid == 0) r = warp_sum(r);
  if (threadIdx.x == 0) sh[0] = r;
  __syncthreads();
  r = sh[0];
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------------------
// Bounded grid barrier for persistent cooperative kernels.
//
// The kernels that use it are launched with cudaLaunchCooperativeKernel, so
// every CTA is resident and the barrier completes.  The spin is still bounded:
// after LAPY_BARRIER_SPIN_LIMIT polls the waiting CTA marks the barrier word
// as failed, records LAPY_ERR_TIMEOUT in *err and leaves; every CTA that
// arrives or polls afterwards sees the mark and returns.
// ---------------------------------------------------------------------------
#ifndef LAPY_BARRIER_SPIN_LIMIT
#define LAPY_BARRIER_SPIN_LIMIT (1u << 26)
#endif

// One 64-bit word, cleared before the launch and alone on its cache line:
// bits 0-31 count arrivals (barrier g completes when they reach (g+1) CTAs),
// bits 32-62 sum the flags the CTAs pass in (so a barrier also tells every
// CTA how many CTAs raised a flag), bit 63 marks a failure.  A CTA whose wait
// times out sets bit 63, which every later poll and arrival sees, and records
// LAPY_ERR_TIMEOUT in *err for the host.
struct GridBarrier {
  unsigned long long* word;
  int* err;  // sticky error flag (0 = ok)
};
constexpr unsigned long long kBarrierFail = 1ull << 63;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_volatile_i32(const int* p) {
  return *((volatile const int*)p);
}

// Barrier over all CTAs of the grid.  *s_flag (shared) is this CTA's flag
// (0 or 1), read and cleared here; *s_seen (shared) receives the flag sum
// (bits 32-62 of the word) when the barrier completed.  Returns false when a
// failure was recorded.  Pass nullptr for both to ignore flags.
__device__ __forceinline__ bool grid_sync(const GridBarrier& b, int* s_flag = nullptr,
                                          unsigned* s_seen = nullptr) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
    unsigned long long add = 1ull;
    if (s_flag) {
      if (*s_flag) add += 1ull << 32;
      *s_flag = 0;
    }
    __threadfence();
    const unsigned long long old = atomicAdd(b.word, add);
    unsigned long long v = old + add;
    bool ok = (old & kBarrierFail) == 0ull;
    const unsigned target = ((unsigned)old / nb + 1u) * nb;
    unsigned spins = 0;
    while (ok && (int)((unsigned)v - target) < 0) {
      if (++spins > LAPY_BARRIER_SPIN_LIMIT) {
        atomicOr(b.word, kBarrierFail);
        atomicCAS(b.err, 0, LAPY_ERR_TIMEOUT);
        ok = false;
        break;
      }
      if (spins > 64) __nanosleep(64);
      v = ld_acquire_u64(b.word);
      if (v & kBarrierFail) ok = false;
    }
    __threadfence();
    if (s_seen) *s_seen = (unsigned)((v >> 32) & 0x7fffffffull);
    s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  return s_ok != 0;
}
