// Heat kernel products of lapy/heat.py:19-111.
//
// H = W S with W the selected rows of the eigenvector matrix (first nev
// columns), squared element-wise for the diagonal K(t, x, x), and S the small
// nev x nt matrix of exp(-lambda t) factors prepared by the caller.  One thread
// per output row; S is staged in shared memory in tiles of kHkRows x kHkCols,
// and each thread keeps kHkCols FP64 accumulators.  The kernel reads W once
// (nrows x nev doubles) and writes H once: HBM-bound for large meshes.
#include "common.cuh"

namespace lapy {

constexpr int kHkThreads = 128;
constexpr int kHkCols = 16;
constexpr int kHkRows = 64;

__global__ void __launch_bounds__(kHkThreads) heat_product_kernel(int64_t nrows, const int64_t* __restrict__ rows,
                                                                  const double* __restrict__ evecs, int64_t ld,
                                                                  int nev, int squared, const double* __restrict__ S,
                                                                  int nt, double* __restrict__ H) {
  __shared__ double st[kHkRows * kHkCols];
  const int64_t r = (int64_t)blockIdx.x * kHkThreads + threadIdx.x;
  const double* w = (r < nrows) ? evecs + (rows ? rows[r] : r) * ld : nullptr;
  for (int j0 = 0; j0 < nt; j0 += kHkCols) {
    const int nc = min(kHkCols, nt - j0);
    double acc[kHkCols];
#pragma unroll
    for (int c = 0; c < kHkCols; ++c) acc[c] = 0.0;
    for (int k0 = 0; k0 < nev; k0 += kHkRows) {
      const int nk = min(kHkRows, nev - k0);
      __syncthreads();
      for (int x = threadIdx.x; x < kHkRows * kHkCols; x += kHkThreads) {
        const int k = x / kHkCols, c = x - k * kHkCols;
        st[x] = (k < nk && c < nc) ? S[(int64_t)(k0 + k) * nt + j0 + c] : 0.0;
      }
      __syncthreads();
      if (w) {
        for (int k = 0; k < nk; ++k) {
          double wk = w[k0 + k];
          if (squared) wk *= wk;
#pragma unroll
          for (int c = 0; c < kHkCols; ++c) acc[c] = fma(wk, st[k * kHkCols + c], acc[c]);
        }
      }
    }
    if (w) {
      double* h = H + r * nt + j0;
#pragma unroll
      for (int c = 0; c < kHkCols; ++c)
        if (c < nc) h[c] = acc[c];
    }
  }
}

}  // namespace lapy

using namespace lapy;

extern "C" int lapy_heat_product_f64(int64_t nrows, const int64_t* rows, const double* evecs, int64_t ld, int nev,
                                     int squared, const double* S, int nt, double* H, void* stream) {
  if (nrows < 0 || nev < 0 || nt < 0 || ld < nev) {
    lapy_set_last_message("heat_product: negative size or ld < nev");
    return LAPY_ERR_INVALID;
  }
  if (nrows == 0 || nt == 0) return LAPY_OK;
  if (!evecs || !H || (nev > 0 && !S)) {
    lapy_set_last_message("heat_product: null pointer");
    return LAPY_ERR_INVALID;
  }
  const int64_t blocks = (nrows + kHkThreads - 1) / kHkThreads;
  heat_product_kernel<<<(unsigned)blocks, kHkThreads, 0, (cudaStream_t)stream>>>(nrows, rows, evecs, ld, nev,
                                                                                  squared ? 1 : 0, S, nt, H);
  return lapy_check_launch("heat_product_kernel");
}
