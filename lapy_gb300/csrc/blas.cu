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

// Per-chunk column sums of x .* y (NC columns, one warp per chunk, every
// lane accumulating all columns of its rows), then per segment the sum of
// its chunks' partials in chunk order: reproducible, and a large segment is
// spread over many CTAs instead of one.
template <int NC>
__global__ void __launch_bounds__(256) chunk_col_dot_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                                            int nchunk, const int32_t* __restrict__ chunk_row,
                                                            double* __restrict__ part) {
  // one warp per chunk (no block barrier): lanes stride the chunk's rows
  const int c = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= nchunk) return;
  const int64_t r0 = chunk_row[c], r1 = chunk_row[c + 1];
  double acc[NC];
#pragma unroll
  for (int q = 0; q < NC; ++q) acc[q] = 0.0;
#pragma unroll 4
  for (int64_t r = r0 + lane; r < r1; r += 32) {
    const double* xr = x + r * NC;
    const double* yr = y + r * NC;
    if constexpr (NC % 2 == 0) {
#pragma unroll
      for (int q = 0; q < NC; q += 2) {
        const double2 a = *reinterpret_cast<const double2*>(xr + q);
        const double2 b = *reinterpret_cast<const double2*>(yr + q);
        acc[q] += a.x * b.x;
        acc[q + 1] += a.y * b.y;
      }
    } else {
      acc[0] += xr[0] * yr[0];
    }
  }
#pragma unroll
  for (int q = 0; q < NC; ++q) {
    const double v = warp_sum(acc[q]);
    if (lane == q) part[(int64_t)c * kChunkScratch + q] = v;
  }
}

// One warp per (segment, column): lane l adds chunks l, l + 32, ... of the
// segment, then a butterfly sum (a fixed order for a given chunk count).
__global__ void seg_sum_chunks_kernel(int nseg, int ncol, const int32_t* __restrict__ seg_chunk,
                                      const double* __restrict__ part, double* __restrict__ out) {
  const int t = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (t >= nseg * ncol) return;
  const int s = t / ncol, q = t - s * ncol;
  double acc = 0.0;
  for (int k = seg_chunk[s] + lane; k < seg_chunk[s + 1]; k += 32) acc += part[(int64_t)k * kChunkScratch + q];
  acc = warp_sum(acc);
  if (lane == 0) out[t] = acc;
}

template <int NC>
static int chunked_dot(const double* x, const double* y, const ChunkTable& ct, double* out, cudaStream_t stream) {
  chunk_col_dot_kernel<NC><<<lapy_ceil_div((int64_t)ct.nchunk * 32, 256), 256, 0, stream>>>(x, y, ct.nchunk,
                                                                                           ct.chunk_row, ct.scratch);
  LAPY_TRY(lapy_check_launch("chunk_col_dot_kernel"));
  seg_sum_chunks_kernel<<<lapy_ceil_div((int64_t)ct.nseg * NC * 32, 128), 128, 0, stream>>>(ct.nseg, NC, ct.seg_chunk,
                                                                                           ct.scratch, out);
  return lapy_check_launch("seg_sum_chunks_kernel");
}

static int seg_dot_any(const double* x, const double* y, int ncol, const ChunkTable& ct, double* out,
                       cudaStream_t stream) {
  if (ct.scratch && ct.nchunk > 0) {
    switch (ncol) {
      case 1: return chunked_dot<1>(x, y, ct, out, stream);
      case 2: return chunked_dot<2>(x, y, ct, out, stream);
      case 4: return chunked_dot<4>(x, y, ct, out, stream);
      case 8: return chunked_dot<8>(x, y, ct, out, stream);
      case 16: return chunked_dot<16>(x, y, ct, out, stream);
      default: break;
    }
  }
  seg_col_norm2_kernel<<<ct.nseg, 256, 0, stream>>>(x, y, ncol, ct.seg_row, out);
  return lapy_check_launch("seg_col_norm2_kernel");
}

int seg_col_norm2(const double* x, int ncol, const ChunkTable& ct, double* out, cudaStream_t stream) {
  return seg_dot_any(x, x, ncol, ct, out, stream);
}

int seg_col_dot(const double* x, const double* y, int ncol, const ChunkTable& ct, double* out, cudaStream_t stream) {
  return seg_dot_any(x, y, ncol, ct, out, stream);
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
