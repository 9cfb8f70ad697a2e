// Batched linear solves with FP64 iterative refinement around FP32 PCG.
#include <cmath>
#include <mutex>
#include <vector>
#include "blas.cuh"
#include "ic0.cuh"
#include "solve.cuh"
#include "spmv.cuh"

namespace lapy {

static size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

size_t ir_workspace_bytes(int64_t n, int p, const ChunkTable& ct, int mixed, int precond, int64_t nagg) {
  const int nseg = ct.nseg;
  size_t b = 0;
  b += a256(sizeof(double) * n * p);            // R64
  b += a256(sizeof(float) * n * p) * 2;         // R32, D32
  b += a256(sizeof(double) * nseg * p) * 2;     // bn2, rn2
  b += a256(sizeof(int32_t) * nseg * p) * 2;    // state, mask
  b += mixed ? pcg_workspace_bytes(n, p, ct, sizeof(float), precond, nagg)
             : pcg_workspace_bytes(n, p, ct, sizeof(double), kPrecJacobi);
  return b + 512;
}

// Reliable updates: fold the FP32 correction in and recompute the FP64
// residual after each tenfold drop of the FP32 residual, checked every 8
// iterations.
constexpr double kReliableDelta = 0.1;
constexpr int kReliableEvery = 8;

__global__ void mask_cols_kernel(float* __restrict__ R, int p, const int32_t* __restrict__ chunk_row,
                                 const int32_t* __restrict__ chunk_seg, const int32_t* __restrict__ mask) {
  const int c = blockIdx.x;
  const int s = chunk_seg[c];
  const int64_t r0 = chunk_row[c], r1 = chunk_row[c + 1];
  for (int64_t i = r0 * p + threadIdx.x; i < r1 * p; i += blockDim.x) {
    const int col = (int)(i % p);
    if (mask[s * p + col]) R[i] = 0.0f;
  }
}

// R -= K X in FP64 (R holds B on entry): the SELL copy when present.
// R = B - K X in FP64 (from the SELL copy in one pass; else B copied, then
// the CSR product subtracted)
static int residual64(const SysMatrix& K, const ChunkTable& ct, int p, const double* X, const double* B, double* R,
                      int G, cudaStream_t stream) {
  if (K.sell64.val && sell_spmm<double>(K.sell64, ct.nunit, ct.unit_row, p, X, R, -1.0, 1.0, stream, B) == LAPY_OK)
    return LAPY_OK;
  LAPY_CUDA_TRY(cudaMemcpyAsync(R, B, sizeof(double) * K.n * p, cudaMemcpyDeviceToDevice, stream));
  return csr_spmm<double>(K.n, K.indptr, K.indices, K.k64, p, X, R, -1.0, 1.0, G, stream);
}

int ir_solve(const SysMatrix& K, const ChunkTable& ct, int p, const double* B, double* X,
             double rtol, int maxiter, int mixed, double inner_rtol, int max_rounds, void* ws,
             size_t ws_bytes, cudaStream_t stream, IrStats* stats, double* relres2_host,
             int32_t* state_host) {
  const int64_t n = K.n;
  const int nsp = ct.nseg * p;
  const int precond = mixed ? K.pc32.kind : kPrecJacobi;
  if (ws_bytes < ir_workspace_bytes(n, p, ct, mixed, precond, mixed ? K.pc32.nagg : 0)) return LAPY_ERR_WORKSPACE;
  char* w = (char*)(((uintptr_t)ws + 255) & ~uintptr_t(255));
  double* R64 = (double*)w; w += a256(sizeof(double) * n * p);
  float* R32 = (float*)w; w += a256(sizeof(float) * n * p);
  float* D32 = (float*)w; w += a256(sizeof(float) * n * p);
  double* bn2 = (double*)w; w += a256(sizeof(double) * nsp);
  double* rn2 = (double*)w; w += a256(sizeof(double) * nsp);
  int32_t* st = (int32_t*)w; w += a256(sizeof(int32_t) * nsp);
  int32_t* mask = (int32_t*)w; w += a256(sizeof(int32_t) * nsp);
  void* pws = w;
  const size_t pws_bytes = ws_bytes - (size_t)(w - (char*)ws);
  const int G = spmm_pick_group(n, K.nnz);

  std::vector<double> hb(nsp), hr(nsp);
  std::vector<int32_t> hst(nsp), hmask(nsp, 0), final_st(nsp, LAPY_OK);
  LAPY_TRY(seg_col_norm2(B, p, ct, bn2, stream));
  LAPY_CUDA_TRY(cudaMemcpyAsync(hb.data(), bn2, sizeof(double) * nsp, cudaMemcpyDeviceToHost, stream));
  IrStats local;
  if (!mixed) {
    int it = 0;
    PcgPrecondDesc<double> pc;
    pc.kind = kPrecJacobi;
    pc.dinv = K.dinv64;
    LAPY_TRY(pcg_solve<double>(n, K.indptr, K.indices, K.k64, nullptr, pc, p, ct, B, X, rtol, maxiter, st, pws,
                               pws_bytes, stream, &it, &K.tuning));
    local.rounds = 1;
    local.pcg_iters = it;
    LAPY_CUDA_TRY(cudaMemcpyAsync(hst.data(), st, sizeof(int32_t) * nsp, cudaMemcpyDeviceToHost, stream));
    LAPY_TRY(residual64(K, ct, p, X, B, R64, G, stream));
    LAPY_TRY(seg_col_norm2(R64, p, ct, rn2, stream));
    LAPY_CUDA_TRY(cudaMemcpyAsync(hr.data(), rn2, sizeof(double) * nsp, cudaMemcpyDeviceToHost, stream));
    LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
    for (int i = 0; i < nsp; ++i) {
      if (hst[i] < 0) final_st[i] = hst[i];
      else if (hb[i] > 0 && !(hr[i] <= rtol * rtol * hb[i] * 1.0000001)) final_st[i] = LAPY_ERR_NOCONV;
      if (relres2_host) relres2_host[i] = hb[i] > 0 ? hr[i] / hb[i] : 0.0;
    }
  } else if (K.reliable && K.pc32.kind == kPrecJacobi) {
    // one launch: FP32 iterations, FP64 solution and residual updates
    int it = 0, updates = 0;
    LAPY_TRY(pcg_solve_ru(n, K.indptr, K.indices, K.k64, K.k32, K.sell32.val ? &K.sell32 : nullptr, K.dinv32, p,
                          ct, B, X, D32, rtol, kReliableDelta, kReliableEvery, maxiter, st, pws, pws_bytes, stream,
                          &it, &updates));
    local.rounds = 1;
    local.pcg_iters = it;
    LAPY_CUDA_TRY(cudaMemcpyAsync(hst.data(), st, sizeof(int32_t) * nsp, cudaMemcpyDeviceToHost, stream));
    LAPY_TRY(residual64(K, ct, p, X, B, R64, G, stream));
    LAPY_TRY(seg_col_norm2(R64, p, ct, rn2, stream));
    LAPY_CUDA_TRY(cudaMemcpyAsync(hr.data(), rn2, sizeof(double) * nsp, cudaMemcpyDeviceToHost, stream));
    LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
    for (int i = 0; i < nsp; ++i) {
      if (hst[i] < 0) final_st[i] = hst[i];
      else if (hb[i] > 0 && !(hr[i] <= rtol * rtol * hb[i] * 1.0000001)) final_st[i] = LAPY_ERR_NOCONV;
      if (relres2_host) relres2_host[i] = hb[i] > 0 ? hr[i] / hb[i] : 0.0;
    }
  } else {
    LAPY_CUDA_TRY(cudaMemsetAsync(X, 0, sizeof(double) * n * p, stream));
    LAPY_CUDA_TRY(cudaMemcpyAsync(R64, B, sizeof(double) * n * p, cudaMemcpyDeviceToDevice, stream));
    LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
    bool done = false;
    for (int i = 0; i < nsp; ++i) hmask[i] = !(hb[i] > 0);
    // per-round FP32 target: at least inner_rtol, but only the reduction still
    // missing (with a factor 4 margin) once the residual is close to rtol
    double round_rtol = inner_rtol;
    for (int round = 0; round < max_rounds && !done; ++round) {
      LAPY_TRY(cast_f64_f32(n * p, R64, R32, stream));
      if (round > 0) {
        LAPY_CUDA_TRY(cudaMemcpyAsync(mask, hmask.data(), sizeof(int32_t) * nsp, cudaMemcpyHostToDevice, stream));
        mask_cols_kernel<<<ct.nchunk, 256, 0, stream>>>(R32, p, ct.chunk_row, ct.chunk_seg, mask);
        LAPY_TRY(lapy_check_launch("mask_cols_kernel"));
      }
      int it = 0;
      PcgPrecondDesc<float> pc = K.pc32;
      if (pc.kind == kPrecJacobi || pc.kind == kPrecTwoLevel) pc.dinv = K.dinv32;
      LAPY_TRY(pcg_solve<float>(n, K.indptr, K.indices, K.k32, K.sell32.val ? &K.sell32 : nullptr, pc, p, ct, R32,
                                D32, round_rtol, maxiter, st, pws, pws_bytes, stream, &it, &K.tuning));
      local.rounds++;
      local.pcg_iters += it;
      LAPY_TRY(add_f32_to_f64(n * p, D32, X, stream));
      LAPY_TRY(residual64(K, ct, p, X, B, R64, G, stream));
      LAPY_TRY(seg_col_norm2(R64, p, ct, rn2, stream));
      LAPY_CUDA_TRY(cudaMemcpyAsync(hr.data(), rn2, sizeof(double) * nsp, cudaMemcpyDeviceToHost, stream));
      LAPY_CUDA_TRY(cudaMemcpyAsync(hst.data(), st, sizeof(int32_t) * nsp, cudaMemcpyDeviceToHost, stream));
      LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
      done = true;
      for (int i = 0; i < nsp; ++i) {
        if (hmask[i]) continue;
        if (hst[i] == LAPY_ERR_NAN || hst[i] == LAPY_ERR_BREAKDOWN || !std::isfinite(hr[i])) {
          final_st[i] = (hst[i] < 0) ? hst[i] : LAPY_ERR_NAN;
          hmask[i] = 1;
          continue;
        }
        if (hr[i] <= rtol * rtol * hb[i]) hmask[i] = 1;
        else done = false;
      }
      double need = 1.0;  // largest remaining reduction factor over active columns
      for (int i = 0; i < nsp; ++i)
        if (!hmask[i] && hr[i] > 0) need = std::min(need, 0.25 * rtol * std::sqrt(hb[i] / hr[i]));
      round_rtol = std::max(inner_rtol, std::min(0.5, need));
    }
    for (int i = 0; i < nsp; ++i) {
      if (final_st[i] == LAPY_OK && hb[i] > 0 && !(hr[i] <= rtol * rtol * hb[i])) final_st[i] = LAPY_ERR_NOCONV;
      if (relres2_host) relres2_host[i] = hb[i] > 0 ? hr[i] / hb[i] : 0.0;
    }
  }
  int worst = LAPY_OK;
  for (int i = 0; i < nsp; ++i) {
    if (state_host) state_host[i] = final_st[i];
    if (final_st[i] != LAPY_OK && worst == LAPY_OK) worst = final_st[i];
  }
  local.status = worst;
  if (stats) *stats = local;
  return LAPY_OK;
}

__global__ void axpby_kernel(int64_t n, double a, const double* __restrict__ x, double b,
                             const double* __restrict__ y, double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = y ? a * x[i] + b * y[i] : a * x[i];
}
int vec_axpby(int64_t nnz, double a, const double* x, double b, const double* y, double* out,
              cudaStream_t stream) {
  if (nnz <= 0) return LAPY_OK;
  axpby_kernel<<<lapy_ceil_div(nnz, 256), 256, 0, stream>>>(nnz, a, x, b, y, out);
  return lapy_check_launch("axpby_kernel");
}

__global__ void add_diag_kernel(int64_t n, const int32_t* __restrict__ pos, double b,
                                const double* __restrict__ d, double* __restrict__ vals) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t k = pos[i];
  if (k >= 0) vals[k] += b * d[i];
}
int add_diag(int64_t n, const int32_t* diag_pos, double b, const double* d, double* vals,
             cudaStream_t stream) {
  add_diag_kernel<<<lapy_ceil_div(n, 256), 256, 0, stream>>>(n, diag_pos, b, d, vals);
  return lapy_check_launch("add_diag_kernel");
}

__global__ void jacobi_kernel(int64_t n, const int32_t* __restrict__ pos, const double* __restrict__ vals,
                              double* __restrict__ d64, float* __restrict__ d32) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t k = pos[i];
  const double v = (k >= 0) ? vals[k] : 0.0;
  const double inv = (v != 0.0 && isfinite(v)) ? 1.0 / v : 1.0;
  if (d64) d64[i] = inv;
  if (d32) d32[i] = (float)inv;
}
int jacobi_inverse(int64_t n, const int32_t* diag_pos, const double* vals, double* dinv64,
                   float* dinv32, cudaStream_t stream) {
  jacobi_kernel<<<lapy_ceil_div(n, 256), 256, 0, stream>>>(n, diag_pos, vals, dinv64, dinv32);
  return lapy_check_launch("jacobi_kernel");
}

}  // namespace lapy

using namespace lapy;

// ---------------------------------------------------------------------------
// C ABI: element-wise matrix combination and the batched PCG solve
// ---------------------------------------------------------------------------
extern "C" int lapy_vec_axpby(int64_t n, double a, const double* x, double b, const double* y,
                              double* out, void* stream) {
  if (n < 0 || !x || !out) return LAPY_ERR_INVALID;
  return vec_axpby(n, a, x, b, y, out, (cudaStream_t)stream);
}

extern "C" int lapy_csr_add_diag(int64_t n, const int32_t* diag_pos, double b, const double* d,
                                 double* vals, void* stream) {
  if (n <= 0 || !diag_pos || !d || !vals) return LAPY_ERR_INVALID;
  return add_diag(n, diag_pos, b, d, vals, (cudaStream_t)stream);
}

static int next_pow2_le16(int c) {
  int p = 1;
  while (p < c && p < 16) p <<= 1;
  return p;
}

static size_t solve_layout(int64_t n, int64_t nnz, int nseg, int ncol, int mixed, int precond, char* base,
                           int32_t** diag_pos, double** dinv64, float** dinv32, float** k32,
                           double** Bp, double** Xp, void** chunk_mem, void** ir_ws, size_t* ir_bytes,
                           void** sell_mem, size_t* sell_bytes, int* nchunk_out, ChunkTable* ct_plan,
                           const int32_t* seg_row) {
  const int w = std::min(ncol, 16);
  const int p = next_pow2_le16(w);
  ChunkTable ct;
  std::vector<int32_t> srow(seg_row, seg_row + nseg + 1);
  plan_chunks(srow.data(), nseg, 4 * lapy_num_sms(), &ct);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* q = base ? base + off : nullptr;
    off += a256(bytes);
    return q;
  };
  char* p0 = take(sizeof(int32_t) * n);
  char* p1 = take(sizeof(double) * n);
  char* p2 = take(sizeof(float) * n);
  char* p3 = take(sizeof(float) * nnz);
  char* p4 = take(sizeof(double) * n * p);
  char* p5 = take(sizeof(double) * n * p);
  char* p6 = take(chunk_table_bytes(ct));
  const size_t irb = ir_workspace_bytes(n, p, ct, mixed, precond);
  char* p7 = take(irb);
  const size_t sellb = mixed ? sell_bytes_bound(nnz, ct, sizeof(float)) : 0;
  char* p8 = take(sellb);
  if (base) {
    *diag_pos = (int32_t*)p0;
    *dinv64 = (double*)p1;
    *dinv32 = (float*)p2;
    *k32 = (float*)p3;
    *Bp = (double*)p4;
    *Xp = (double*)p5;
    *chunk_mem = p6;
    *ir_ws = p7;
    *ir_bytes = irb;
    *sell_mem = p8;
    *sell_bytes = sellb;
    *nchunk_out = ct.nchunk;
    *ct_plan = ct;
  }
  return off + 256;
}

extern "C" size_t lapy_pcg_solve_workspace_bytes(int64_t n, int64_t nnz, int nseg, const int32_t* seg_row,
                                                 int ncol, int mixed) {
  if (n <= 0 || nnz <= 0 || nseg <= 0 || !seg_row || ncol <= 0) return 0;
  return solve_layout(n, nnz, nseg, ncol, mixed, kPrecJacobi, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                      nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, seg_row);
}

// Padding allowance of the SELL copies of a triangular factor (slices take the
// longest row of 32; the lower half of a mesh pattern has rows of 1 to ~8).
constexpr double kFactorPad = 3.0;

// Two SELL copies (G and G') of the lower / upper halves of an n x n pattern
// with nnz entries, on the PCG's unit table.
static size_t factor_sell_bytes(int64_t n, int64_t nnz, int nseg, const int32_t* seg_row) {
  ChunkTable ct;
  std::vector<int32_t> srow(seg_row, seg_row + nseg + 1);
  plan_chunks(srow.data(), nseg, 4 * lapy_num_sms(), &ct);
  return 2 * sell_bytes_bound((nnz + n) / 2, ct, sizeof(float), kFactorPad) + 512;
}

// Device memory of the IC(0) preconditioner of an n-row system: level plan,
// FP64 factor, its FP32 copy, 1 / L[i][i] and a pivot counter.
static size_t ic0_pre_bytes(int64_t n, int64_t nnz) {
  return ic0_plan_bytes(n) + a256(8 * (size_t)nnz) + a256(4 * (size_t)nnz) + a256(4 * (size_t)n) + a256(64) + 256;
}

// Shared body of the PCG entry points; `factored` (may be null) selects the
// factored preconditioner z = G' (G r) with FP32 factors on CSR patterns;
// `ic0` the IC(0) preconditioner, factored here (*ic0_fixed: pivots replaced).
static int pcg_solve_impl(int64_t n, const int32_t* indptr, const int32_t* indices, const double* k_vals,
                          int64_t nnz, int nseg, const int32_t* seg_row, int ncol, const double* b, double* x,
                          double rtol, int maxiter, int mixed, double inner_rtol, int32_t* status_out,
                          double* relres_out, int64_t* iters_out, void* ws, size_t ws_bytes, cudaStream_t stream,
                          const PcgPrecondDesc<float>* factored, bool ic0 = false, int32_t* ic0_fixed = nullptr) {
  const int precond = factored ? kPrecFactored : ic0 ? kPrecIC0 : kPrecJacobi;
  if (ic0 && !mixed) {
    lapy_set_last_message("pcg_solve: the IC(0) preconditioner runs inside the mixed-precision solve");
    return LAPY_ERR_INVALID;
  }
  if (n <= 0 || !indptr || !indices || !k_vals || nnz <= 0 || nseg <= 0 || !seg_row || ncol <= 0 ||
      !b || !x || !(rtol > 0) || maxiter <= 0 || !ws) {
    lapy_set_last_message("pcg_solve: invalid arguments");
    return LAPY_ERR_INVALID;
  }
  if (seg_row[0] != 0 || seg_row[nseg] != n) {
    lapy_set_last_message("pcg_solve: segment rows must span [0, n)");
    return LAPY_ERR_INVALID;
  }
  const size_t main_bytes = solve_layout(n, nnz, nseg, ncol, mixed, precond, nullptr, nullptr, nullptr, nullptr,
                                         nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                         nullptr, nullptr, seg_row);
  if (ws_bytes < main_bytes + (factored ? factor_sell_bytes(n, nnz, nseg, seg_row) : 0) +
                     (ic0 ? ic0_pre_bytes(n, nnz) : 0))
    return LAPY_ERR_WORKSPACE;
  int32_t* diag_pos;
  double *dinv64, *Bp, *Xp;
  float *dinv32, *k32;
  void *chunk_mem, *ir_ws, *sell_mem;
  size_t ir_bytes, sell_bytes;
  int nchunk;
  ChunkTable ct;
  char* base = (char*)(((uintptr_t)ws + 255) & ~uintptr_t(255));
  solve_layout(n, nnz, nseg, ncol, mixed, precond, base, &diag_pos, &dinv64, &dinv32, &k32, &Bp, &Xp, &chunk_mem,
               &ir_ws, &ir_bytes, &sell_mem, &sell_bytes, &nchunk, &ct, seg_row);
  LAPY_TRY(upload_chunk_table(&ct, chunk_mem, stream));
  LAPY_TRY(lapy_csr_diag_index(n, indptr, indices, diag_pos, stream));
  LAPY_TRY(jacobi_inverse(n, diag_pos, k_vals, dinv64, dinv32, stream));
  if (mixed) LAPY_TRY(cast_f64_f32(nnz, k_vals, k32, stream));
  SysMatrix K;
  K.n = n;
  K.nnz = nnz;
  K.indptr = indptr;
  K.indices = indices;
  K.k64 = k_vals;
  K.k32 = k32;
  K.dinv64 = dinv64;
  K.dinv32 = dinv32;
  if (factored) {
    // SELL copies of G and G' on the PCG's units (CSR when they do not fit)
    K.pc32 = *factored;
    const size_t gsb = sell_bytes_bound((nnz + n) / 2, ct, sizeof(float), kFactorPad);
    char* gmem = base + a256(main_bytes);
    bool fits = false;
    LAPY_TRY(build_sell<float>(n, factored->g_ptr, factored->g_idx, factored->g_val, ct, gmem, gsb, &K.pc32.g_sell,
                               &fits, stream));
    if (!fits) K.pc32.g_sell = SellMatrix<float>();
    LAPY_TRY(build_sell<float>(n, factored->gt_ptr, factored->gt_idx, factored->gt_val, ct, gmem + gsb, gsb,
                               &K.pc32.gt_sell, &fits, stream));
    if (!fits) K.pc32.gt_sell = SellMatrix<float>();
  }
  if (ic0) {
    char* w = base + a256(main_bytes);
    const size_t pb = ic0_plan_bytes(n);
    Ic0Plan plan;
    LAPY_TRY(ic0_plan(n, indptr, indices, w, pb, &plan, stream));
    char* w2 = (char*)(((uintptr_t)w + 255) & ~uintptr_t(255)) + pb;
    double* L64 = (double*)w2; w2 += a256(8 * (size_t)nnz);
    float* L32 = (float*)w2; w2 += a256(4 * (size_t)nnz);
    float* dinv_ic = (float*)w2; w2 += a256(4 * (size_t)n);
    unsigned* fixed_dev = (unsigned*)w2;
    LAPY_CUDA_TRY(cudaMemsetAsync(L64, 0, 8 * (size_t)nnz, stream));
    LAPY_TRY(ic0_factor(plan, indptr, indices, k_vals, L64, fixed_dev, stream));
    LAPY_TRY(ic0_to_f32(plan, L64, nnz, L32, dinv_ic, stream));
    unsigned fx = 0;
    LAPY_CUDA_TRY(cudaMemcpyAsync(&fx, fixed_dev, sizeof(fx), cudaMemcpyDeviceToHost, stream));
    LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
    if (ic0_fixed) *ic0_fixed = (int32_t)fx;
    PcgPrecondDesc<float> pc;
    pc.kind = kPrecIC0;
    pc.dinv = dinv_ic;
    pc.ic_val = L32;
    pc.ic_diag = plan.diag_pos;
    pc.ic_nlev_f = plan.nlev_f;
    pc.ic_nlev_b = plan.nlev_b;
    pc.ic_lev_f_ptr = plan.lev_f_ptr;
    pc.ic_lev_f_row = plan.lev_f_row;
    pc.ic_lev_b_ptr = plan.lev_b_ptr;
    pc.ic_lev_b_row = plan.lev_b_row;
    K.pc32 = pc;
  }
  if (mixed) {
    bool fits = false;
    LAPY_TRY(build_sell<float>(n, indptr, indices, k32, ct, sell_mem, sell_bytes, &K.sell32, &fits, stream));
    if (!fits) K.sell32 = SellMatrix<float>();
  }
  int64_t total_iters = 0;
  for (int c0 = 0; c0 < ncol; c0 += 16) {
    const int w = std::min(16, ncol - c0);
    const int p = next_pow2_le16(w);
    LAPY_TRY(pack_cols(n, b, ncol, c0, w, p, Bp, stream));
    std::vector<double> rr(nseg * p);
    std::vector<int32_t> st(nseg * p);
    IrStats stats;
    LAPY_TRY(ir_solve(K, ct, p, Bp, Xp, rtol, maxiter, mixed, inner_rtol, 12, ir_ws, ir_bytes, stream, &stats,
                      rr.data(), st.data()));
    total_iters += stats.pcg_iters;
    LAPY_TRY(unpack_cols(n, Xp, p, w, x, ncol, c0, stream));
    for (int s = 0; s < nseg; ++s)
      for (int c = 0; c < w; ++c) {
        if (status_out) status_out[(int64_t)s * ncol + c0 + c] = st[s * p + c];
        if (relres_out) relres_out[(int64_t)s * ncol + c0 + c] = std::sqrt(rr[s * p + c]);
      }
  }
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  if (iters_out) *iters_out = total_iters;
  return LAPY_OK;
}

extern "C" int lapy_pcg_solve(int64_t n, const int32_t* indptr, const int32_t* indices,
                              const double* k_vals, int64_t nnz, int nseg, const int32_t* seg_row,
                              int ncol, const double* b, double* x, double rtol, int maxiter, int mixed,
                              double inner_rtol, int32_t* status_out, double* relres_out,
                              int64_t* iters_out, void* ws, size_t ws_bytes, void* stream) {
  return pcg_solve_impl(n, indptr, indices, k_vals, nnz, nseg, seg_row, ncol, b, x, rtol, maxiter, mixed,
                        inner_rtol, status_out, relres_out, iters_out, ws, ws_bytes, (cudaStream_t)stream, nullptr);
}

extern "C" size_t lapy_spai_pcg_workspace_bytes(int64_t n, int64_t nnz, int nseg, const int32_t* seg_row,
                                                int ncol) {
  if (n <= 0 || nnz <= 0 || nseg <= 0 || !seg_row || ncol <= 0) return 0;
  return a256(solve_layout(n, nnz, nseg, ncol, 1, kPrecFactored, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                           nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, seg_row)) +
         factor_sell_bytes(n, nnz, nseg, seg_row) + 256;
}

extern "C" int lapy_spai_pcg_solve(int64_t n, const int32_t* indptr, const int32_t* indices, const double* k_vals,
                                   int64_t nnz, int nseg, const int32_t* seg_row, int ncol, const double* b,
                                   double* x, double rtol, int maxiter, double inner_rtol, const int32_t* lptr,
                                   const int32_t* lcol, const float* g_lower, const int32_t* uptr,
                                   const int32_t* ucol, const float* g_upper, int32_t* status_out,
                                   double* relres_out, int64_t* iters_out, void* ws, size_t ws_bytes,
                                   void* stream) {
  if (!lptr || !lcol || !g_lower || !uptr || !ucol || !g_upper) {
    lapy_set_last_message("spai_pcg_solve: missing factor arrays");
    return LAPY_ERR_INVALID;
  }
  PcgPrecondDesc<float> pc;
  pc.kind = kPrecFactored;
  pc.g_ptr = lptr;
  pc.g_idx = lcol;
  pc.g_val = g_lower;
  pc.gt_ptr = uptr;
  pc.gt_idx = ucol;
  pc.gt_val = g_upper;
  return pcg_solve_impl(n, indptr, indices, k_vals, nnz, nseg, seg_row, ncol, b, x, rtol, maxiter, 1, inner_rtol,
                        status_out, relres_out, iters_out, ws, ws_bytes, (cudaStream_t)stream, &pc);
}

extern "C" size_t lapy_ic0_pcg_workspace_bytes(int64_t n, int64_t nnz, int nseg, const int32_t* seg_row, int ncol) {
  if (n <= 0 || nnz <= 0 || nseg <= 0 || !seg_row || ncol <= 0) return 0;
  return a256(solve_layout(n, nnz, nseg, ncol, 1, kPrecIC0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                           nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, seg_row)) +
         ic0_pre_bytes(n, nnz) + 256;
}

extern "C" int lapy_ic0_pcg_solve(int64_t n, const int32_t* indptr, const int32_t* indices, const double* k_vals,
                                  int64_t nnz, int nseg, const int32_t* seg_row, int ncol, const double* b,
                                  double* x, double rtol, int maxiter, double inner_rtol, int32_t* status_out,
                                  double* relres_out, int64_t* iters_out, int32_t* n_fixed, void* ws,
                                  size_t ws_bytes, void* stream) {
  return pcg_solve_impl(n, indptr, indices, k_vals, nnz, nseg, seg_row, ncol, b, x, rtol, maxiter, 1, inner_rtol,
                        status_out, relres_out, iters_out, ws, ws_bytes, (cudaStream_t)stream, nullptr, true,
                        n_fixed);
}

// ---------------------------------------------------------------------------
// Allocation-free variant of lapy_pcg_solve.
//
// For callers that cannot allocate device memory: processes whose device
// memory is fully reserved by another allocator, code paths where a device
// allocation is not allowed, or plain C callers that do not manage a
// workspace.  Its scratch is this file-scope device array (held by every GPU
// that loads the library, until the process exits); its address is looked up
// once per device with cudaGetSymbolAddress, on the first call made with that
// device current.  The looked-up address is kept for the life of the process: after a
// cudaDeviceReset of a device, this entry point must not be called on it
// again (the module is reloaded and the kept address is stale).  Like
// lapy_pcg_solve, the call returns after the solve has finished on `stream`.
// Every call shares the one array and leaves its contents behind; the solve
// clears everything it needs zeroed itself.  Calls that overlap on the GPU
// (two streams, or two host threads) race on the array.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_pcg_static_scratch[LAPY_STATIC_SCRATCH_BYTES];

static int static_scratch_address(void** out) {
  static std::mutex mu;
  static std::vector<void*> per_device;
  int dev = 0;
  LAPY_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if ((int)per_device.size() <= dev) per_device.resize(dev + 1, nullptr);
  if (per_device[dev] == nullptr) {
    void* ptr = nullptr;
    LAPY_CUDA_TRY(cudaGetSymbolAddress(&ptr, g_pcg_static_scratch));
    per_device[dev] = ptr;
  }
  *out = per_device[dev];
  return LAPY_OK;
}

extern "C" int lapy_pcg_solve_static(int64_t n, const int32_t* indptr, const int32_t* indices,
                                     const double* k_vals, int64_t nnz, int nseg, const int32_t* seg_row,
                                     int ncol, const double* b, double* x, double rtol, int maxiter, int mixed,
                                     double inner_rtol, int32_t* status_out, double* relres_out,
                                     int64_t* iters_out, void* stream) {
  if (n <= 0 || !indptr || !indices || !k_vals || nnz <= 0 || nseg <= 0 || !seg_row || ncol <= 0 ||
      !b || !x || !(rtol > 0) || maxiter <= 0) {
    lapy_set_last_message("pcg_solve_static: invalid arguments");
    return LAPY_ERR_INVALID;
  }
  if (seg_row[0] != 0 || seg_row[nseg] != n) {
    lapy_set_last_message("pcg_solve_static: segment rows must span [0, n)");
    return LAPY_ERR_INVALID;
  }
  const size_t need = lapy_pcg_solve_workspace_bytes(n, nnz, nseg, seg_row, ncol, mixed);
  if (need == 0 || need > LAPY_STATIC_SCRATCH_BYTES) {
    lapy_set_last_message("pcg_solve_static: this problem needs %zu bytes of scratch; the static array "
                          "holds %zu (LAPY_STATIC_SCRATCH_BYTES); use lapy_pcg_solve with a workspace",
                          need, (size_t)LAPY_STATIC_SCRATCH_BYTES);
    return LAPY_ERR_WORKSPACE;
  }
  void* ws = nullptr;
  LAPY_TRY(static_scratch_address(&ws));
  return lapy_pcg_solve(n, indptr, indices, k_vals, nnz, nseg, seg_row, ncol, b, x, rtol, maxiter, mixed,
                        inner_rtol, status_out, relres_out, iters_out, ws, LAPY_STATIC_SCRATCH_BYTES, stream);
}
