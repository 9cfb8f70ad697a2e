// Incomplete Cholesky IC(0): level plan, factorization and triangular solves.
#pragma once
#include <vector>
#include "common.cuh"

namespace lapy {

// Level plan of a CSR pattern (sorted columns, full diagonal): rows grouped
// by their forward level (factorization and L^-1) and backward level (L^-T).
struct Ic0Plan {
  int64_t n = 0;
  int nlev_f = 0, nlev_b = 0;
  int32_t* diag_pos = nullptr;   // device, n
  int32_t* lev_f_ptr = nullptr;  // device, nlev_f + 1
  int32_t* lev_f_row = nullptr;  // device, n
  int32_t* lev_b_ptr = nullptr;  // device, nlev_b + 1
  int32_t* lev_b_row = nullptr;  // device, n
  std::vector<int32_t> h_lev_f_ptr, h_lev_b_ptr;
};

// Stored in the workspace after a factorization, so that apply calls find
// the plan without host state.
struct Ic0PlanHeader {
  uint32_t magic;
  int64_t n;
  int32_t nlev_f, nlev_b;
};
constexpr uint32_t kIc0Magic = 0x1c0a11u;

// Device bytes of a plan of n rows (including the header slot at its end).
size_t ic0_plan_bytes(int64_t n);
// Build the plan into `mem` (pattern copied to the host for the level sets).
int ic0_plan(int64_t n, const int32_t* indptr, const int32_t* indices, void* mem, size_t bytes, Ic0Plan* plan,
             cudaStream_t stream);
// L (lower part, with the upper part mirrored) of the matrix kv on the plan's
// pattern; *nfixed_dev counts replaced pivots.
int ic0_factor(const Ic0Plan& plan, const int32_t* indptr, const int32_t* indices, const double* kv, double* L,
               unsigned* nfixed_dev, cudaStream_t stream);
// z = (L L')^-1 r for ncol row-major columns (y: n x ncol scratch).
int ic0_apply(const Ic0Plan& plan, const int32_t* indptr, const int32_t* indices, const double* L, int ncol,
              const double* r, double* y, double* z, cudaStream_t stream);

// FP32 copy of L and dinv32[i] = 1 / L[i][i] for the FP32 PCG iterations.
int ic0_to_f32(const Ic0Plan& plan, const double* L64, int64_t nnz, float* L32, float* dinv32, cudaStream_t stream);

}  // namespace lapy
