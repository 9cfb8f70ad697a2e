// Small vector kernels shared by the solvers (segmented norms, casts, packing).
#pragma once
#include "common.cuh"
#include "pcg.cuh"

namespace lapy {

// out[s*ncol + c] = sum over rows of segment s of x[row*ncol + c]^2 (per-chunk partials in the
// chunk table's scratch, then per segment in chunk order)
int seg_col_norm2(const double* x, int ncol, const ChunkTable& ct, double* out, cudaStream_t stream);
// out[s*ncol + c] = sum over segment s's rows of x(row, c) * y(row, c)
int seg_col_dot(const double* x, const double* y, int ncol, const ChunkTable& ct, double* out, cudaStream_t stream);
// y = (float) x
int cast_f64_f32(int64_t n, const double* x, float* y, cudaStream_t stream);
// x64 += (double) d32
int add_f32_to_f64(int64_t n, const float* d, double* x, cudaStream_t stream);
// dst (n x w) <- src columns [c0, c0+w) of an n x ncol array, zero-padded to wpad columns
int pack_cols(int64_t n, const double* src, int ncol, int c0, int w, int wpad, double* dst, cudaStream_t stream);
int unpack_cols(int64_t n, const double* src, int wpad, int w, double* dst, int ncol, int c0, cudaStream_t stream);

}  // namespace lapy
