// CSR sparse x dense (row-major n x ncol) products.
#pragma once
#include "common.cuh"
#include "pcg.cuh"

namespace lapy {

// Lanes per row picked from the mean row length (4..32).
int spmm_pick_group(int64_t n, int64_t nnz);

template <typename V>
int csr_spmm(int64_t n, const int32_t* indptr, const int32_t* indices, const V* vals, int ncol,
             const V* x, V* y, V alpha, V beta, int group, cudaStream_t stream);

// Group-of-G-lanes-per-row accumulation of sum_k vals[k] * x[cols[k]*ncol + c]
// for NC consecutive columns starting at c0; the result is in lane 0..G-1
// after the butterfly (every lane holds the full sums).  All lanes of the
// warp must call it (invalid rows pass valid=false).
template <typename V, typename XV, int G, int NC>
__device__ __forceinline__ void row_dot_group(const int32_t* __restrict__ indptr,
                                              const int32_t* __restrict__ indices,
                                              const V* __restrict__ vals, const XV* __restrict__ x,
                                              int ncol, int c0, int nc, int64_t row, bool valid,
                                              int lg, V acc[NC]) {
#pragma unroll
  for (int q = 0; q < NC; ++q) acc[q] = V(0);
  const int32_t k0 = valid ? indptr[row] : 0, k1 = valid ? indptr[row + 1] : 0;
  for (int32_t k = k0 + lg; k < k1; k += G) {
    const V a = vals[k];
    const int64_t base = (int64_t)indices[k] * ncol + c0;
#pragma unroll
    for (int q = 0; q < NC; ++q)
      if (q < nc) acc[q] += a * (V)x[base + q];
  }
#pragma unroll
  for (int q = 0; q < NC; ++q) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o, G);
  }
}

// Y = alpha * Mat * X + beta * B from a SELL copy (B = Y when null; one warp
// per 32-row unit, lane = row; ncol in {1, 2, 4, 8, 16}).  Returns
// LAPY_ERR_INVALID for other widths (callers then use csr_spmm).
template <typename V>
int sell_spmm(const SellMatrix<V>& M, int nunit, const int32_t* unit_row, int ncol, const V* x, V* y, V alpha,
              V beta, cudaStream_t stream, const V* b = nullptr);

}  // namespace lapy
