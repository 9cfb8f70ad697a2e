// Deterministic exclusive scan: per-tile scan -> scan of tile sums -> add.
#include "scan.cuh"

namespace lapy {

__device__ __forceinline__ int32_t block_exclusive_scan(int32_t v, int32_t* sh, int32_t* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int32_t s = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    sh[lane] = s;  // inclusive warp totals
  }
  __syncthreads();
  const int32_t warp_off = wid ? sh[wid - 1] : 0;
  *total = sh[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_off + x - v;
}

__global__ void scan_tiles_kernel(const int32_t* __restrict__ in, int32_t* __restrict__ out,
                                  int64_t n, int32_t* __restrict__ tile_sums) {
  __shared__ int32_t sh[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int32_t v[kScanItems];
  int32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < n) ? in[base + k] : 0;
    s += v[k];
  }
  int32_t total;
  int32_t off = block_exclusive_scan(s, sh, &total);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = off;
    off += v[k];
  }
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// One block scans the tile sums in place (exclusive) and writes the total.
__global__ void scan_tile_sums_kernel(int32_t* sums, int64_t ntiles, int32_t* total_out) {
  __shared__ int32_t sh[32];
  int32_t carry = 0;
  for (int64_t b = 0; b < ntiles; b += blockDim.x) {
    const int64_t i = b + threadIdx.x;
    const int32_t v = (i < ntiles) ? sums[i] : 0;
    int32_t tot;
    const int32_t ex = block_exclusive_scan(v, sh, &tot);
    if (i < ntiles) sums[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) *total_out = carry;
}

__global__ void scan_add_kernel(int32_t* out, int64_t n, const int32_t* tile_offsets) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += tile_offsets[i / kScanTile];
}

int exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, int32_t* scratch,
                       cudaStream_t stream) {
  if (n <= 0) {
    LAPY_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(int32_t), stream));
    return LAPY_OK;
  }
  const unsigned ntiles = lapy_ceil_div(n, kScanTile);
  scan_tiles_kernel<<<ntiles, kScanThreads, 0, stream>>>(in, out, n, scratch);
  LAPY_TRY(lapy_check_launch("scan_tiles_kernel"));
  scan_tile_sums_kernel<<<1, kScanThreads, 0, stream>>>(scratch, ntiles, out + n);
  LAPY_TRY(lapy_check_launch("scan_tile_sums_kernel"));
  if (ntiles > 1) {
    scan_add_kernel<<<lapy_ceil_div(n, 256), 256, 0, stream>>>(out, n, scratch);
    LAPY_TRY(lapy_check_launch("scan_add_kernel"));
  }
  return LAPY_OK;
}

}  // namespace lapy
