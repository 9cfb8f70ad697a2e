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
void lapy_profile_add_pcg(double ms, long long iters, long long rows, long long nnz, int p, int elem_bytes);
void lapy_profile_add_reorth(long long steps, long long second_passes);

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
// after LAPY_BARRIER_SPIN_LIMIT polls the waiting CTA records LAPY_ERR_TIMEOUT
// in *err and leaves; every CTA checks *err after each barrier and returns.
// ---------------------------------------------------------------------------
#ifndef LAPY_BARRIER_SPIN_LIMIT
#define LAPY_BARRIER_SPIN_LIMIT (1u << 26)
#endif

struct GridBarrier {
  unsigned int* count;  // arrivals in the current generation
  unsigned int* gen;    // generation counter
  int* err;             // sticky error flag (0 = ok)
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_volatile_i32(const int* p) {
  return *((volatile const int*)p);
}

// Returns true when the grid may continue, false when an error was recorded.
__device__ __forceinline__ bool grid_sync(const GridBarrier& b) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
    const unsigned my_gen = ld_acquire_u32(b.gen);
    __threadfence();
    const unsigned arrived = atomicAdd(b.count, 1u);
    if (arrived == nblocks - 1) {
      atomicExch(b.count, 0u);
      __threadfence();
      atomicAdd(b.gen, 1u);
    } else {
      unsigned spins = 0;
      while (ld_acquire_u32(b.gen) == my_gen) {
        if (++spins > LAPY_BARRIER_SPIN_LIMIT) {
          atomicCAS(b.err, 0, LAPY_ERR_TIMEOUT);
          break;
        }
        if (spins > 64) __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ld_volatile_i32(b.err) == 0;
}
