// Incomplete Cholesky IC(0) of an SPD CSR matrix on the device.
//
// The reference factors its systems exactly (SuperLU: lapy/solver.py:707-712,
// lapy/heat.py:226); IC(0) is the classical incomplete fallback for the same
// SPD systems.  Row i of L is computed from the rows j < i it references, so
// rows are grouped into levels (level of i = 1 + the largest level of its
// lower neighbours; mesh matrices in their subdivision order have 8), and the
// factorization and the forward solve proceed level by level with one thread
// per row.  The backward solve uses the reverse levels.  L is kept on the
// matrix's own pattern: its lower part (columns <= row) holds L and its upper
// part the mirror L[j][i] of every entry (i, j), j > i, so both triangular
// solves read rows.
//
// Arithmetic follows the textbook row-wise IC(0) exactly (sums in ascending
// column order, no fused multiply-add: this file is compiled with
// --fmad=false), so the factor equals a straightforward CPU restatement to the
// last bit.  A pivot that is not positive is replaced by the matrix diagonal
// and counted.
#include <algorithm>
#include <cmath>
#include <vector>
#include "common.cuh"
#include "ic0.cuh"
#include "scan.cuh"

namespace lapy {

static size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

size_t ic0_plan_bytes(int64_t n) {
  return a256(4 * (size_t)n) + 2 * (a256(4 * (size_t)(n + 1)) + a256(4 * (size_t)n)) + a256(64);
}

int ic0_plan(int64_t n, const int32_t* indptr, const int32_t* indices, void* mem, size_t bytes, Ic0Plan* plan,
             cudaStream_t stream) {
  if (bytes < ic0_plan_bytes(n)) return LAPY_ERR_WORKSPACE;
  char* w = (char*)(((uintptr_t)mem + 255) & ~uintptr_t(255));
  plan->diag_pos = (int32_t*)w; w += a256(4 * (size_t)n);
  plan->lev_f_ptr = (int32_t*)w; w += a256(4 * (size_t)(n + 1));
  plan->lev_f_row = (int32_t*)w; w += a256(4 * (size_t)n);
  plan->lev_b_ptr = (int32_t*)w; w += a256(4 * (size_t)(n + 1));
  plan->lev_b_row = (int32_t*)w; w += a256(4 * (size_t)n);
  plan->n = n;
  std::vector<int32_t> hptr(n + 1);
  LAPY_CUDA_TRY(cudaMemcpyAsync(hptr.data(), indptr, 4 * (size_t)(n + 1), cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  const int64_t nnz = hptr[n];
  std::vector<int32_t> hidx(nnz);
  LAPY_CUDA_TRY(cudaMemcpyAsync(hidx.data(), indices, 4 * (size_t)nnz, cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  std::vector<int32_t> diag(n, -1), lf(n, 0), lb(n, 0);
  for (int64_t i = 0; i < n; ++i) {
    int32_t prev = -1;
    for (int32_t k = hptr[i]; k < hptr[i + 1]; ++k) {
      const int32_t j = hidx[k];
      if (j < 0 || j >= n || j <= prev) {
        lapy_set_last_message("ic0: row %lld: column indices must be in range and strictly ascending", (long long)i);
        return LAPY_ERR_INVALID;
      }
      prev = j;
      if (j == i) diag[i] = k;
      else if (j < i) lf[i] = std::max(lf[i], lf[j] + 1);
    }
    if (diag[i] < 0) {
      lapy_set_last_message("ic0: row %lld has no diagonal entry", (long long)i);
      return LAPY_ERR_INVALID;
    }
  }
  for (int64_t i = n - 1; i >= 0; --i)
    for (int32_t k = hptr[i]; k < hptr[i + 1]; ++k)
      if (hidx[k] > i) lb[i] = std::max(lb[i], lb[hidx[k]] + 1);
  // rows grouped by level (ascending rows inside a level)
  auto group = [&](const std::vector<int32_t>& lev, std::vector<int32_t>& ptr, std::vector<int32_t>& row) {
    const int nl = n > 0 ? *std::max_element(lev.begin(), lev.end()) + 1 : 0;
    ptr.assign(nl + 1, 0);
    for (int64_t i = 0; i < n; ++i) ++ptr[lev[i] + 1];
    for (int l = 0; l < nl; ++l) ptr[l + 1] += ptr[l];
    row.resize(n);
    std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
    for (int64_t i = 0; i < n; ++i) row[fill[lev[i]]++] = (int32_t)i;
    return nl;
  };
  std::vector<int32_t> fptr, frow, bptr, brow;
  plan->nlev_f = group(lf, fptr, frow);
  plan->nlev_b = group(lb, bptr, brow);
  plan->h_lev_f_ptr = fptr;
  plan->h_lev_b_ptr = bptr;
  LAPY_CUDA_TRY(cudaMemcpyAsync(plan->diag_pos, diag.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, stream));
  LAPY_CUDA_TRY(cudaMemcpyAsync(plan->lev_f_ptr, fptr.data(), 4 * fptr.size(), cudaMemcpyHostToDevice, stream));
  LAPY_CUDA_TRY(cudaMemcpyAsync(plan->lev_f_row, frow.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, stream));
  LAPY_CUDA_TRY(cudaMemcpyAsync(plan->lev_b_ptr, bptr.data(), 4 * bptr.size(), cudaMemcpyHostToDevice, stream));
  LAPY_CUDA_TRY(cudaMemcpyAsync(plan->lev_b_row, brow.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, stream));
  // the host vectors are pageable: the copies complete before they go away
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  return LAPY_OK;
}

// Rows of one level, one thread per row: L[i][j] for the lower entries in
// ascending j, then the pivot.
__global__ void ic0_factor_level_kernel(int32_t r0, int32_t r1, const int32_t* __restrict__ lev_row,
                                        const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                        const double* __restrict__ kv, const int32_t* __restrict__ diag_pos,
                                        double* __restrict__ L, unsigned* __restrict__ nfixed) {
  for (int32_t t = r0 + blockIdx.x * blockDim.x + threadIdx.x; t < r1; t += gridDim.x * blockDim.x) {
    const int32_t i = lev_row[t];
    const int32_t k0 = indptr[i], kd = diag_pos[i];
    for (int32_t k = k0; k < kd; ++k) {
      const int32_t j = indices[k];
      double acc = 0.0;
      int32_t a = k0, b = indptr[j];
      const int32_t be = diag_pos[j];
      while (a < k && b < be) {  // columns m < j present in both rows, ascending
        const int32_t ca = indices[a], cb = indices[b];
        if (ca == cb) {
          acc = acc + L[a] * L[b];
          ++a;
          ++b;
        } else if (ca < cb) {
          ++a;
        } else {
          ++b;
        }
      }
      L[k] = (kv[k] - acc) / L[be];
    }
    double acc = 0.0;
    for (int32_t k = k0; k < kd; ++k) acc = acc + L[k] * L[k];
    double d = kv[kd] - acc;
    if (!(d > 0.0) || !isfinite(d)) {
      d = kv[kd];
      atomicAdd(nfixed, 1u);
    }
    L[kd] = sqrt(d);
  }
}

// Upper entries (i, j), j > i, receive L[j][i] (binary search in row j's
// lower part).
__global__ void ic0_mirror_kernel(int64_t n, const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                  const int32_t* __restrict__ diag_pos, double* __restrict__ L) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int32_t k = diag_pos[i] + 1; k < indptr[i + 1]; ++k) {
    const int32_t j = indices[k];
    int32_t lo = indptr[j], hi = diag_pos[j] - 1;
    double v = 0.0;
    while (lo <= hi) {
      const int32_t mid = (lo + hi) >> 1;
      const int32_t c = indices[mid];
      if (c == (int32_t)i) {
        v = L[mid];
        break;
      }
      if (c < (int32_t)i) lo = mid + 1;
      else hi = mid - 1;
    }
    L[k] = v;
  }
}

// Forward (lower = true: y = L^-1 r) or backward (z = L^-T y) solve of the
// rows of one level; ncol columns, row-major.
template <bool LOWER>
__global__ void ic0_solve_level_kernel(int32_t r0, int32_t r1, const int32_t* __restrict__ lev_row,
                                       const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                       const int32_t* __restrict__ diag_pos, const double* __restrict__ L, int ncol,
                                       const double* __restrict__ in, double* __restrict__ out) {
  for (int32_t t = r0 + blockIdx.x * blockDim.x + threadIdx.x; t < r1; t += gridDim.x * blockDim.x) {
    const int32_t i = lev_row[t];
    const int32_t kd = diag_pos[i];
    const int32_t kb = LOWER ? indptr[i] : kd + 1, ke = LOWER ? kd : indptr[i + 1];
    const double dinv = 1.0 / L[kd];
    for (int c = 0; c < ncol; ++c) {
      double acc = in[(int64_t)i * ncol + c];
      for (int32_t k = kb; k < ke; ++k) acc = acc - L[k] * out[(int64_t)indices[k] * ncol + c];
      out[(int64_t)i * ncol + c] = acc * dinv;
    }
  }
}

int ic0_factor(const Ic0Plan& plan, const int32_t* indptr, const int32_t* indices, const double* kv, double* L,
               unsigned* nfixed_dev, cudaStream_t stream) {
  const int64_t n = plan.n;
  LAPY_CUDA_TRY(cudaMemsetAsync(nfixed_dev, 0, sizeof(unsigned), stream));
  for (int l = 0; l < plan.nlev_f; ++l) {
    const int32_t r0 = plan.h_lev_f_ptr[l], r1 = plan.h_lev_f_ptr[l + 1];
    ic0_factor_level_kernel<<<std::max(1u, lapy_ceil_div(r1 - r0, 256)), 256, 0, stream>>>(
        r0, r1, plan.lev_f_row, indptr, indices, kv, plan.diag_pos, L, nfixed_dev);
    LAPY_TRY(lapy_check_launch("ic0_factor_level_kernel"));
  }
  ic0_mirror_kernel<<<std::max(1u, lapy_ceil_div(n, 256)), 256, 0, stream>>>(n, indptr, indices, plan.diag_pos, L);
  return lapy_check_launch("ic0_mirror_kernel");
}

int ic0_apply(const Ic0Plan& plan, const int32_t* indptr, const int32_t* indices, const double* L, int ncol,
              const double* r, double* y, double* z, cudaStream_t stream) {
  for (int l = 0; l < plan.nlev_f; ++l) {
    const int32_t r0 = plan.h_lev_f_ptr[l], r1 = plan.h_lev_f_ptr[l + 1];
    ic0_solve_level_kernel<true><<<std::max(1u, lapy_ceil_div(r1 - r0, 256)), 256, 0, stream>>>(
        r0, r1, plan.lev_f_row, indptr, indices, plan.diag_pos, L, ncol, r, y);
    LAPY_TRY(lapy_check_launch("ic0_solve_level_kernel"));
  }
  for (int l = 0; l < plan.nlev_b; ++l) {
    const int32_t r0 = plan.h_lev_b_ptr[l], r1 = plan.h_lev_b_ptr[l + 1];
    ic0_solve_level_kernel<false><<<std::max(1u, lapy_ceil_div(r1 - r0, 256)), 256, 0, stream>>>(
        r0, r1, plan.lev_b_row, indptr, indices, plan.diag_pos, L, ncol, y, z);
    LAPY_TRY(lapy_check_launch("ic0_solve_level_kernel"));
  }
  return LAPY_OK;
}

__global__ void ic0_to_f32_kernel(int64_t n, int64_t nnz, const double* __restrict__ L64,
                                  const int32_t* __restrict__ diag_pos, float* __restrict__ L32,
                                  float* __restrict__ dinv32) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nnz) L32[t] = (float)L64[t];
  if (t < n) dinv32[t] = (float)(1.0 / L64[diag_pos[t]]);
}

int ic0_to_f32(const Ic0Plan& plan, const double* L64, int64_t nnz, float* L32, float* dinv32, cudaStream_t stream) {
  const int64_t m = std::max<int64_t>(nnz, plan.n);
  ic0_to_f32_kernel<<<lapy_ceil_div(m, 256), 256, 0, stream>>>(plan.n, nnz, L64, plan.diag_pos, L32, dinv32);
  return lapy_check_launch("ic0_to_f32_kernel");
}

}  // namespace lapy

using namespace lapy;

// Workspace of lapy_ic0_factor / lapy_ic0_apply: the level plan (kept from
// the factor call for the apply calls) and the intermediate of the solves.
extern "C" size_t lapy_ic0_workspace_bytes(int64_t n, int64_t nnz, int ncol) {
  if (n <= 0 || nnz <= 0 || ncol <= 0) return 0;
  return ic0_plan_bytes(n) + a256(8 * (size_t)n * ncol) + a256(sizeof(Ic0PlanHeader)) + 512;
}

namespace {
// Host copy of a plan stored in the workspace (the level pointers are also
// kept there, after the device arrays, so apply calls need no host state).
int load_plan(int64_t n, void* work, Ic0Plan* plan, cudaStream_t stream) {
  char* base = (char*)(((uintptr_t)work + 255) & ~uintptr_t(255));
  char* w = base;
  plan->n = n;
  plan->diag_pos = (int32_t*)w; w += a256(4 * (size_t)n);
  plan->lev_f_ptr = (int32_t*)w; w += a256(4 * (size_t)(n + 1));
  plan->lev_f_row = (int32_t*)w; w += a256(4 * (size_t)n);
  plan->lev_b_ptr = (int32_t*)w; w += a256(4 * (size_t)(n + 1));
  plan->lev_b_row = (int32_t*)w; w += a256(4 * (size_t)n);
  Ic0PlanHeader h;
  LAPY_CUDA_TRY(cudaMemcpyAsync(&h, base + ic0_plan_bytes(n) - a256(64), sizeof(h), cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  if (h.magic != kIc0Magic || h.n != n) {
    lapy_set_last_message("ic0_apply: the workspace holds no plan of this matrix (call lapy_ic0_factor first)");
    return LAPY_ERR_INVALID;
  }
  plan->nlev_f = h.nlev_f;
  plan->nlev_b = h.nlev_b;
  plan->h_lev_f_ptr.resize(h.nlev_f + 1);
  plan->h_lev_b_ptr.resize(h.nlev_b + 1);
  LAPY_CUDA_TRY(cudaMemcpyAsync(plan->h_lev_f_ptr.data(), plan->lev_f_ptr, 4 * (size_t)(h.nlev_f + 1),
                                cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaMemcpyAsync(plan->h_lev_b_ptr.data(), plan->lev_b_ptr, 4 * (size_t)(h.nlev_b + 1),
                                cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  return LAPY_OK;
}
}  // namespace

extern "C" int lapy_ic0_factor(int64_t n, const int32_t* indptr, const int32_t* indices, const double* k_vals,
                               int64_t nnz, double* l_vals, int32_t* n_fixed, int32_t* n_levels, void* work,
                               size_t ws_bytes, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n <= 0 || nnz <= 0 || !indptr || !indices || !k_vals || !l_vals || !work) {
    lapy_set_last_message("ic0_factor: invalid arguments");
    return LAPY_ERR_INVALID;
  }
  if (ws_bytes < lapy_ic0_workspace_bytes(n, nnz, 1)) return LAPY_ERR_WORKSPACE;
  Ic0Plan plan;
  LAPY_TRY(ic0_plan(n, indptr, indices, work, ws_bytes, &plan, stream));
  char* base = (char*)(((uintptr_t)work + 255) & ~uintptr_t(255));
  Ic0PlanHeader h{kIc0Magic, n, plan.nlev_f, plan.nlev_b};
  char* hdr = base + ic0_plan_bytes(n) - a256(64);
  unsigned* fixed_dev = (unsigned*)(hdr + 32);
  LAPY_CUDA_TRY(cudaMemcpyAsync(hdr, &h, sizeof(h), cudaMemcpyHostToDevice, stream));
  LAPY_CUDA_TRY(cudaMemsetAsync(l_vals, 0, 8 * (size_t)nnz, stream));
  LAPY_TRY(ic0_factor(plan, indptr, indices, k_vals, l_vals, fixed_dev, stream));
  unsigned fx = 0;
  LAPY_CUDA_TRY(cudaMemcpyAsync(&fx, fixed_dev, sizeof(fx), cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  if (n_fixed) *n_fixed = (int32_t)fx;
  if (n_levels) {
    n_levels[0] = plan.nlev_f;
    n_levels[1] = plan.nlev_b;
  }
  return LAPY_OK;
}

extern "C" int lapy_ic0_apply(int64_t n, const int32_t* indptr, const int32_t* indices, const double* l_vals,
                              int64_t nnz, int ncol, const double* r, double* z, void* work, size_t ws_bytes,
                              void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n <= 0 || nnz <= 0 || ncol <= 0 || !indptr || !indices || !l_vals || !r || !z || !work) {
    lapy_set_last_message("ic0_apply: invalid arguments");
    return LAPY_ERR_INVALID;
  }
  if (ws_bytes < lapy_ic0_workspace_bytes(n, nnz, ncol)) return LAPY_ERR_WORKSPACE;
  Ic0Plan plan;
  LAPY_TRY(load_plan(n, work, &plan, stream));
  char* base = (char*)(((uintptr_t)work + 255) & ~uintptr_t(255));
  double* y = (double*)(base + ic0_plan_bytes(n));
  LAPY_TRY(ic0_apply(plan, indptr, indices, l_vals, ncol, r, y, z, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  return LAPY_OK;
}
