// CSR SpMV / SpMM with G lanes per row (G chosen from the mean row length).
#include "spmv.cuh"

namespace lapy {

int spmm_pick_group(int64_t n, int64_t nnz) {
  const double avg = n > 0 ? (double)nnz / (double)n : 1.0;
  if (avg <= 6.0) return 4;
  if (avg <= 12.0) return 8;
  if (avg <= 24.0) return 16;
  return 32;
}

template <typename V, int G, int NC>
__global__ void __launch_bounds__(256) spmm_kernel(int64_t n, const int32_t* __restrict__ indptr,
                                                   const int32_t* __restrict__ indices,
                                                   const V* __restrict__ vals, int ncol,
                                                   const V* __restrict__ x, V* __restrict__ y,
                                                   V alpha, V beta) {
  const int lg = threadIdx.x & (G - 1);
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int c0 = blockIdx.y * NC;
  const int nc = min(NC, ncol - c0);
  const bool valid = row < n;
  V acc[NC];
  row_dot_group<V, V, G, NC>(indptr, indices, vals, x, ncol, c0, nc, row, valid, lg, acc);
  if (!valid) return;
  // lane q of the group writes column q (q < nc); for NC > G lanes loop.
  for (int q = lg; q < nc; q += G) {
    V v = V(0);
#pragma unroll
    for (int qq = 0; qq < NC; ++qq)
      if (qq == q) v = acc[qq];
    const int64_t o = row * ncol + c0 + q;
    y[o] = (beta == V(0)) ? alpha * v : alpha * v + beta * y[o];
  }
}

template <typename V, int G>
static int launch_spmm_g(int64_t n, const int32_t* indptr, const int32_t* indices, const V* vals,
                         int ncol, const V* x, V* y, V alpha, V beta, cudaStream_t stream) {
  const unsigned blocks = lapy_ceil_div(n * G, 256);
  if (ncol == 1) {
    spmm_kernel<V, G, 1><<<dim3(blocks, 1), 256, 0, stream>>>(n, indptr, indices, vals, ncol, x, y, alpha, beta);
  } else if (ncol <= 4) {
    spmm_kernel<V, G, 4><<<dim3(blocks, 1), 256, 0, stream>>>(n, indptr, indices, vals, ncol, x, y, alpha, beta);
  } else {
    spmm_kernel<V, G, 8><<<dim3(blocks, lapy_ceil_div(ncol, 8)), 256, 0, stream>>>(n, indptr, indices, vals,
                                                                                 ncol, x, y, alpha, beta);
  }
  return lapy_check_launch("spmm_kernel");
}

// Many columns (ncol > 8, e.g. the final Rayleigh-Ritz block): one thread per
// (row, group of 8 columns), the row's entries walked once per group with
// eight accumulators, so each gathered row of X is read 8 values at a time
// (groups of lanes per row reduced through shuffles cost more here).
template <typename V>
__global__ void __launch_bounds__(256) spmm_rowcols_kernel(int64_t n, const int32_t* __restrict__ indptr,
                                                           const int32_t* __restrict__ indices,
                                                           const V* __restrict__ vals, int ncol,
                                                           const V* __restrict__ x, V* __restrict__ y, V alpha,
                                                           V beta) {
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  const int c0 = blockIdx.y * 8;
  const int nc = min(8, ncol - c0);
  V acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = V(0);
  for (int32_t k = indptr[row]; k < indptr[row + 1]; ++k) {
    const V a = __ldg(vals + k);
    const V* xr = x + (int64_t)__ldg(indices + k) * ncol + c0;
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (q < nc) acc[q] += a * __ldg(xr + q);
  }
  V* yr = y + row * ncol + c0;
#pragma unroll
  for (int q = 0; q < 8; ++q)
    if (q < nc) yr[q] = (beta == V(0)) ? alpha * acc[q] : alpha * acc[q] + beta * yr[q];
}

template <typename V>
int csr_spmm(int64_t n, const int32_t* indptr, const int32_t* indices, const V* vals, int ncol,
             const V* x, V* y, V alpha, V beta, int group, cudaStream_t stream) {
  if (n <= 0 || ncol <= 0) return LAPY_OK;
  if (ncol > 8) {
    spmm_rowcols_kernel<V><<<dim3(lapy_ceil_div(n, 256), lapy_ceil_div(ncol, 8)), 256, 0, stream>>>(
        n, indptr, indices, vals, ncol, x, y, alpha, beta);
    return lapy_check_launch("spmm_rowcols_kernel");
  }
  switch (group) {
    case 4: return launch_spmm_g<V, 4>(n, indptr, indices, vals, ncol, x, y, alpha, beta, stream);
    case 8: return launch_spmm_g<V, 8>(n, indptr, indices, vals, ncol, x, y, alpha, beta, stream);
    case 16: return launch_spmm_g<V, 16>(n, indptr, indices, vals, ncol, x, y, alpha, beta, stream);
    case 32: return launch_spmm_g<V, 32>(n, indptr, indices, vals, ncol, x, y, alpha, beta, stream);
    default: return LAPY_ERR_INVALID;
  }
}

template int csr_spmm<double>(int64_t, const int32_t*, const int32_t*, const double*, int, const double*,
                              double*, double, double, int, cudaStream_t);
template int csr_spmm<float>(int64_t, const int32_t*, const int32_t*, const float*, int, const float*,
                             float*, float, float, int, cudaStream_t);

__global__ void diag_mm_kernel(int64_t n, const double* __restrict__ d, int ncol,
                               const double* __restrict__ x, double* __restrict__ y, double alpha,
                               double beta) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * ncol) return;
  const double v = alpha * d[i / ncol] * x[i];
  y[i] = (beta == 0.0) ? v : v + beta * y[i];
}


// ---- SELL (sliced ELL, 32-row slices) product, lane = row -----------------
template <typename V, int NP>
__global__ void __launch_bounds__(256) sell_spmm_kernel(int nunit, const int32_t* __restrict__ unit_row,
                                                        const int32_t* __restrict__ slice_ptr,
                                                        const int32_t* __restrict__ col, const V* __restrict__ val,
                                                        const V* __restrict__ x, const V* __restrict__ b,
                                                        V* __restrict__ y, V alpha, V beta) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < nunit; u += nw) {
    const int32_t base = slice_ptr[u];
    const int w = (slice_ptr[u + 1] - base) >> 5;
    V acc[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) acc[q] = V(0);
#pragma unroll 4
    for (int k = 0; k < w; ++k) {
      const V a = __ldg(val + base + 32 * k + lane);
      const V* xr = x + (int64_t)__ldg(col + base + 32 * k + lane) * NP;
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] += a * __ldg(xr + q);
    }
    const int64_t row = unit_row[u] + lane;
    if (row < unit_row[u + 1]) {
      V* yr = y + row * NP;
      const V* br = b ? b + row * NP : yr;  // y = alpha A x + beta b (b = y when null)
#pragma unroll
      for (int q = 0; q < NP; ++q) yr[q] = (beta == V(0)) ? alpha * acc[q] : alpha * acc[q] + beta * br[q];
    }
  }
}

template <typename V>
int sell_spmm(const SellMatrix<V>& M, int nunit, const int32_t* unit_row, int ncol, const V* x, V* y, V alpha,
              V beta, cudaStream_t stream, const V* b) {
  if (!M.val || nunit <= 0) return LAPY_ERR_INVALID;
  const unsigned grid = std::min<unsigned>(lapy_ceil_div((int64_t)nunit * 32, 256), 8u * lapy_num_sms());
#define LAPY_SELL_CASE(NPV)                                                                                  \
  case NPV:                                                                                                \
    sell_spmm_kernel<V, NPV><<<grid, 256, 0, stream>>>(nunit, unit_row, M.slice_ptr, M.col, M.val, x, b, y, alpha, \
                                                       beta);                                              \
    return lapy_check_launch("sell_spmm_kernel");
  switch (ncol) {
    LAPY_SELL_CASE(1)
    LAPY_SELL_CASE(2)
    LAPY_SELL_CASE(4)
    LAPY_SELL_CASE(8)
    LAPY_SELL_CASE(16)
    default:
      return LAPY_ERR_INVALID;
  }
#undef LAPY_SELL_CASE
}

template int sell_spmm<double>(const SellMatrix<double>&, int, const int32_t*, int, const double*, double*, double,
                               double, cudaStream_t, const double*);
template int sell_spmm<float>(const SellMatrix<float>&, int, const int32_t*, int, const float*, float*, float, float,
                              cudaStream_t, const float*);

}  // namespace lapy

using namespace lapy;

static int spmm_args_ok(int64_t n, const int32_t* indptr, const int32_t* indices, const void* vals,
                        int ncol, const void* x, const void* y, int group) {
  if (n <= 0 || !indptr || !indices || !vals || ncol <= 0 || !x || !y) return 0;
  if (group != 0 && group != 4 && group != 8 && group != 16 && group != 32) return 0;
  if (x == y) return 0;
  return 1;
}

extern "C" int lapy_csr_spmm_f64(int64_t n, const int32_t* indptr, const int32_t* indices,
                                 const double* vals, int ncol, const double* x, double* y,
                                 double alpha, double beta, int group, void* stream) {
  if (!spmm_args_ok(n, indptr, indices, vals, ncol, x, y, group)) {
    lapy_set_last_message("csr_spmm_f64: invalid arguments");
    return LAPY_ERR_INVALID;
  }
  if (group == 0) {
    int32_t nnz = 0;
    LAPY_CUDA_TRY(cudaMemcpyAsync(&nnz, indptr + n, sizeof(int32_t), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    LAPY_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    group = spmm_pick_group(n, nnz);
  }
  return csr_spmm<double>(n, indptr, indices, vals, ncol, x, y, alpha, beta, group, (cudaStream_t)stream);
}

extern "C" int lapy_csr_spmm_f32(int64_t n, const int32_t* indptr, const int32_t* indices,
                                 const float* vals, int ncol, const float* x, float* y, float alpha,
                                 float beta, int group, void* stream) {
  if (!spmm_args_ok(n, indptr, indices, vals, ncol, x, y, group)) {
    lapy_set_last_message("csr_spmm_f32: invalid arguments");
    return LAPY_ERR_INVALID;
  }
  if (group == 0) {
    int32_t nnz = 0;
    LAPY_CUDA_TRY(cudaMemcpyAsync(&nnz, indptr + n, sizeof(int32_t), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    LAPY_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    group = spmm_pick_group(n, nnz);
  }
  return csr_spmm<float>(n, indptr, indices, vals, ncol, x, y, alpha, beta, group, (cudaStream_t)stream);
}

extern "C" int lapy_diag_mm_f64(int64_t n, const double* d, int ncol, const double* x, double* y,
                                double alpha, double beta, void* stream) {
  if (n <= 0 || !d || ncol <= 0 || !x || !y || x == y) return LAPY_ERR_INVALID;
  diag_mm_kernel<<<lapy_ceil_div(n * ncol, 256), 256, 0, (cudaStream_t)stream>>>(n, d, ncol, x, y, alpha, beta);
  return lapy_check_launch("diag_mm_kernel");
}
