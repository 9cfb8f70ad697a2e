#include "blas.cuh"

namespace lapy {

__global__ void seg_col_norm2_kernel(const double* __restrict__ x, const double* __restrict__ y, int ncol,
                                     const int32_t* __restrict__ seg_row, double* __restrict__ out) {
  __shared__ double sh[32];
  const int s = blockIdx.x;
  const int64_t r0 = seg_row[s], r1 = seg_row[s + 1];
  for (int c = 0; c < ncol; ++c) {
    double acc = 0.0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
      acc += x[r * ncol + c] * y[r * ncol + c];
    }
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) out[(int64_t)s * ncol + c] = acc;
  }
}

int seg_col_norm2(const double* x, int ncol, const ChunkTable& ct, double* out, cudaStream_t stream) {
  seg_col_norm2_kernel<<<ct.nseg, 256, 0, stream>>>(x, x, ncol, ct.seg_row, out);
  return lapy_check_launch("seg_col_norm2_kernel");
}

int seg_col_dot(const double* x, const double* y, int ncol, const ChunkTable& ct, double* out, cudaStream_t stream) {
  seg_col_norm2_kernel<<<ct.nseg, 256, 0, stream>>>(x, y, ncol, ct.seg_row, out);
  return lapy_check_launch("seg_col_norm2_kernel");
}

__global__ void cast_kernel(int64_t n, const double* __restrict__ x, float* __restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = (float)x[i];
}
int cast_f64_f32(int64_t n, const double* x, float* y, cudaStream_t stream) {
  if (n <= 0) return LAPY_OK;
  cast_kernel<<<lapy_ceil_div(n, 256), 256, 0, stream>>>(n, x, y);
  return lapy_check_launch("cast_kernel");
}

__global__ void add32_kernel(int64_t n, const float* __restrict__ d, double* __restrict__ x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] += (double)d[i];
}
int add_f32_to_f64(int64_t n, const float* d, double* x, cudaStream_t stream) {
  if (n <= 0) return LAPY_OK;
  add32_kernel<<<lapy_ceil_div(n, 256), 256, 0, stream>>>(n, d, x);
  return lapy_check_launch("add32_kernel");
}

__global__ void pack_kernel(int64_t n, const double* __restrict__ src, int ncol, int c0, int w, int wpad,
                            double* __restrict__ dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * wpad) return;
  const int64_t r = i / wpad;
  const int c = (int)(i - r * wpad);
  dst[i] = (c < w) ? src[r * ncol + c0 + c] : 0.0;
}
int pack_cols(int64_t n, const double* src, int ncol, int c0, int w, int wpad, double* dst, cudaStream_t stream) {
  pack_kernel<<<lapy_ceil_div(n * wpad, 256), 256, 0, stream>>>(n, src, ncol, c0, w, wpad, dst);
  return lapy_check_launch("pack_kernel");
}

__global__ void unpack_kernel(int64_t n, const double* __restrict__ src, int wpad, int w,
                              double* __restrict__ dst, int ncol, int c0) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * w) return;
  const int64_t r = i / w;
  const int c = (int)(i - r * w);
  dst[r * ncol + c0 + c] = src[r * wpad + c];
}
int unpack_cols(int64_t n, const double* src, int wpad, int w, double* dst, int ncol, int c0, cudaStream_t stream) {
  unpack_kernel<<<lapy_ceil_div(n * w, 256), 256, 0, stream>>>(n, src, wpad, w, dst, ncol, c0);
  return lapy_check_launch("unpack_kernel");
}

}  // namespace lapy
