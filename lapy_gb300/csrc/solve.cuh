// Linear solves K X = B on a batch of segments: FP64 PCG, or FP32 PCG inside
// FP64 iterative refinement (residuals recomputed in FP64 each round).
#pragma once
#include "pcg.cuh"

namespace lapy {

struct SysMatrix {
  int64_t n = 0;
  int64_t nnz = 0;
  const int32_t* indptr = nullptr;
  const int32_t* indices = nullptr;
  const double* k64 = nullptr;
  const float* k32 = nullptr;
  const double* dinv64 = nullptr;
  const float* dinv32 = nullptr;
  PcgPrecondDesc<float> pc32;  // kind == kPrecFactored selects the learned/SPAI factor
  SellMatrix<float> sell32;    // SELL copy of k32 (val == nullptr: CSR path)
  SellMatrix<double> sell64;   // SELL copy of k64 for the FP64 residuals (optional)
  // mixed solves: one reliable-update PCG launch (true, Jacobi only) or
  // restarted FP32 refinement rounds (false).  Keeping the CG direction
  // across residual replacements stagnates on some right-hand sides (FP32
  // iterates), so the restarted rounds are the default.
  bool reliable = false;
  PcgTuning tuning;            // launch knobs of the persistent PCG
};

struct IrStats {
  int rounds = 0;
  int64_t pcg_iters = 0;
  int status = LAPY_OK;
};

size_t ir_workspace_bytes(int64_t n, int p, const ChunkTable& ct, int mixed, int precond, int64_t nagg = 0);

// Solve K X = B for p columns (p in {1,2,4,8,16}); X overwritten.  On return
// relres2[s*p + c] holds ||B - K X||^2 / ||B||^2 (0 for zero columns) and
// state[s*p + c] the outcome (LAPY_OK or a negative status).
int ir_solve(const SysMatrix& K, const ChunkTable& ct, int p, const double* B, double* X,
             double rtol, int maxiter, int mixed, double inner_rtol, int max_rounds, void* ws,
             size_t ws_bytes, cudaStream_t stream, IrStats* stats, double* relres2_host,
             int32_t* state_host);

// out = a*x + b*y on nnz values; y may be null.
int vec_axpby(int64_t nnz, double a, const double* x, double b, const double* y, double* out,
              cudaStream_t stream);
// vals[diag_pos[i]] += b * d[i]
int add_diag(int64_t n, const int32_t* diag_pos, double b, const double* d, double* vals,
             cudaStream_t stream);
// dinv = 1/vals[diag_pos] (f64 and f32 copies; missing/zero diagonal -> 1)
int jacobi_inverse(int64_t n, const int32_t* diag_pos, const double* vals, double* dinv64,
                   float* dinv32, cudaStream_t stream);

}  // namespace lapy
